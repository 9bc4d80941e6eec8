// CPU checks of hsspack_gb300/csrc/host_util.h (built and run by
// tests/test_host_util.py): MDSTEDC's split test decides like the reference's
// expression, and the host fill / scatter of packed eigenvectors writes
// exactly rows 0..n-1 of every column.
#include "host_util.h"

#include <cstdio>
#include <random>

using namespace hss;

static int fails = 0;
#define CHECK(c)                                                          \
  do {                                                                    \
    if (!(c)) {                                                           \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c);             \
      ++fails;                                                            \
    }                                                                     \
  } while (0)

// the reference's test, mdstedc.f90: TINY = EPS*SQRT(|D(i)|)*SQRT(|D(i+1)|)
static bool reference(double e, double a, double b) {
  return !(std::fabs(e) > HSS_EPS * std::sqrt(std::fabs(a)) * std::sqrt(std::fabs(b)));
}

static int2 rows(int x, int y) {
  int2 r;
  r.x = x;
  r.y = y;
  return r;
}

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0), ex(-320.0, 300.0), k(-8.0, 8.0);
  long long mism = 0, near = 0;
  for (int i = 0; i < 2000000; ++i) {
    const double a = u(rng) * std::pow(10.0, ex(rng) / (i % 3 == 0 ? 1.0 : 4.0));
    const double b = u(rng) * std::pow(10.0, ex(rng) / (i % 5 == 0 ? 1.0 : 4.0));
    double e;
    if (i % 2 == 0) {  // at the boundary, a few ulps either side
      e = HSS_EPS * std::sqrt(std::fabs(a)) * std::sqrt(std::fabs(b)) *
          (1.0 + std::floor(k(rng)) * 2.220446049250313e-16);
      ++near;
    } else {
      e = u(rng) * std::pow(10.0, ex(rng) / 4.0);
    }
    mism += negligible(e, a, b) != reference(e, a, b);
  }
  CHECK(mism == 0);
  CHECK(negligible(0.0, 1.0, 1.0) && !negligible(1.0, 1.0, 1.0));
  CHECK(negligible(1e-300, 0.0, 5.0) == reference(1e-300, 0.0, 5.0));

  // packed scatter into n = 37 columns of leading dimension 41
  {
    const int n = 37;
    const long long ld = 41;
    std::vector<double> z((size_t)ld * n, 7.0), src;
    PackedZ pz;
    pz.seg.resize(n);
    pz.off.assign(n + 1, 0);
    for (int j = 0; j < n; ++j) {
      const int x = (j * 5) % n, y = std::min(n, x + j % 7);
      pz.seg[j] = rows(x, y);
      pz.off[j + 1] = pz.off[j] + (y - x);
      for (int i = x; i < y; ++i) src.push_back(1000.0 * j + i);
    }
    pz.total = pz.off[n];
    {
      HostFill f(z.data(), n, ld, true);
      CHECK(f.active());
      f.finish(&pz, src.data());
    }
    for (int j = 0; j < n; ++j)
      for (long long i = 0; i < ld; ++i) {
        const double want = i >= n ? 7.0
                            : (i >= pz.seg[j].x && i < pz.seg[j].y) ? 1000.0 * j + i
                                                                    : 0.0;
        CHECK(z[j * ld + i] == want);
      }
  }
  // the dense path (no packed data) and a fill released only by the
  // destructor leave zeros; an inactive fill touches nothing
  {
    std::vector<double> z(64 * 64, 3.0), w(64 * 64, 3.0), v(64 * 64, 3.0);
    {
      HostFill f(z.data(), 64, 64, true);
      f.finish(nullptr, nullptr);
    }
    { HostFill g(w.data(), 64, 64, true); }
    {
      HostFill h(v.data(), 64, 64, false);
      CHECK(!h.active());
    }
    for (size_t i = 0; i < z.size(); ++i) {
      CHECK(z[i] == 0.0);
      CHECK(w[i] == 0.0);
      CHECK(v[i] == 3.0);
    }
  }
  std::printf("%s: %lld boundary cases\n", fails ? "FAILED" : "OK", near);
  return fails ? 1 : 0;
}
