// host_util.h -- host-side helpers of the C ABI's host entry points that
// need no GPU: MDSTEDC's split test, and the zero-fill / scatter of
// eigenvectors bound for host memory.  Plain C++ (CUDA's vector types only),
// so the CPU tests compile and check them directly.
#pragma once
#include <vector_types.h>

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#ifndef HSS_EPS
#define HSS_EPS 1.1102230246251565e-16 /* 2^-53, LAPACK DLAMCH('Epsilon') */
#endif

namespace hss {

// MDSTEDC's split test (mdstedc.f90: |E(i)| <= EPS sqrt|D(i)| sqrt|D(i+1)|).
// Squares decide it without square roots unless they are within a relative
// 1e-12 of the boundary or outside the range where they are exact enough;
// those cases take the reference's own expression, so the decision is the
// same.
inline bool negligible(double e, double a, double b) {
  const double ae = std::fabs(e), aa = std::fabs(a), ab = std::fabs(b);
  if (ae > 1e-100 && ae < 1e100 && aa > 1e-100 && aa < 1e100 && ab > 1e-100 && ab < 1e100) {
    const double lhs = ae * ae, rhs = (HSS_EPS * HSS_EPS) * (aa * ab);
    if (lhs > rhs * (1.0 + 1e-12)) return false;
    if (lhs < rhs * (1.0 - 1e-12)) return true;
  }
  return !(ae > HSS_EPS * std::sqrt(aa) * std::sqrt(ab));
}

// MDLASD20 (SRC/mdlasd20.f90:122-300): deflation of the updating problem
// M = [diag(f); z^T] (f ascending).  A small z_j deflates f_j; two poles closer
// than the tolerance are rotated so that the first one's z vanishes (the
// rotation acts on rows p, q of V^T: x <- c x + s y, y <- c y - s x).  On return
// f[0..K) holds the non-deflated poles and f[K..n) the deflated values in the
// reference's order (last deflated first); z[0..K) the non-deflated weights
// (z[K..n) as the rotations left them at their original positions); idxp[j] is
// the original position of new position j (V^T row j of the output is row
// idxp[j] of the rotated input).  Deviations, both readings of undefined
// behaviour in the Fortran: the local ALPHA and BETA that enter the tolerance
// are never set there and count as 0 here, and HFLAG (uninitialised in
// SvdHssUpdat, set .FALSE. only when K > 10) is always .FALSE., i.e. all rows
// are permuted.
struct SvdUpdRot {
  int p, q;
  double c, s;
};
struct SvdUpdDeflation {
  int K = 0;
  double tol = 0.0;
  std::vector<int> idxp;
  std::vector<SvdUpdRot> rot;
};
inline SvdUpdDeflation svdupd_deflate(int n, double *f, double *z) {
  SvdUpdDeflation r;
  r.idxp.assign(n, 0);
  if (n <= 0) return r;
  const double tol = 8.0 * HSS_EPS * std::max(std::fabs(f[n - 1]), std::fabs(f[0]));
  r.tol = tol;
  std::vector<double> ww(n, 0.0);
  int K = 0, K2 = n, jprev = -1;
  for (int j = 0; j < n; ++j) {
    if (std::fabs(z[j]) <= tol) {
      r.idxp[--K2] = j;  // deflated by a small z
    } else {
      jprev = j;
      break;
    }
  }
  if (jprev >= 0) {
    for (int j = jprev + 1; j < n; ++j) {
      if (std::fabs(z[j]) <= tol) {
        r.idxp[--K2] = j;
      } else if (std::fabs(f[j] - f[jprev]) <= tol) {  // close poles: rotate
        const double tau = std::hypot(z[j], z[jprev]);
        const double c = z[j] / tau, s = -z[jprev] / tau;
        z[j] = tau;
        z[jprev] = 0.0;
        r.rot.push_back(SvdUpdRot{jprev, j, c, s});
        r.idxp[--K2] = jprev;
        jprev = j;
      } else {
        ww[K] = z[jprev];
        r.idxp[K++] = jprev;
        jprev = j;
      }
    }
    ww[K] = z[jprev];
    r.idxp[K++] = jprev;
  }
  for (int j = 0; j < K; ++j) z[j] = ww[j];
  for (int j = 0; j < n; ++j) ww[j] = f[r.idxp[j]];
  for (int j = 0; j < n; ++j) f[j] = ww[j];
  if (std::fabs(z[0]) <= tol) z[0] = tol;
  r.K = K;
  return r;
}

// Eigenvectors bound for host memory (mdstedc_): when the columns' supports
// cover little of Z, the solve leaves them packed on the device (the
// supported rows of every output column back to back) instead of writing the
// full n x n matrix; the host zero-fills Z meanwhile and scatters the segments.
struct PackedZ {
  bool want = false;           // request (single problem, supports tracked)
  bool packed = false;         // result: the packed form was produced
  long long total = 0;         // packed doubles
  std::vector<int2> seg;       // per output column: rows [x, y)
  std::vector<long long> off;  // per output column: offset into the packed data
  double *dbuf = nullptr;      // device packed data
};

// Host threads for the output work of the host entry points: all cores but
// two (the solve's own host thread keeps running meanwhile).
inline int host_threads() {
  const unsigned h = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(16u, h > 2 ? h - 2 : 1u));
}

// Zeroes rows 0..n-1 of the n columns of a host matrix (leading dimension ld)
// on worker threads, each owning a range of columns; finish() hands them the
// packed segments (or none), which each worker copies into its own columns
// once they are zeroed, and waits for them (the destructor releases and
// joins them on any other path).
class HostFill {
 public:
  HostFill(double *z, int n, long long ld, bool on) : z_(z), n_(n), ld_(ld) {
    if (!on) return;
    nt_ = host_threads();
    for (int t = 0; t < nt_; ++t) {
      try {
        th_.emplace_back([this, t] { run(t); });
      } catch (...) {
        inline_.push_back(t);  // no thread available: finish() runs this share
      }
    }
    on_ = true;
  }
  bool active() const { return on_; }
  void finish(const PackedZ *pz, const double *src) {
    if (!on_ || done_) return;
    {
      std::lock_guard<std::mutex> g(mu_);
      pz_ = pz;
      src_ = src;
      ready_ = true;
    }
    cv_.notify_all();
    for (int t : inline_) run(t);
    for (auto &x : th_)
      if (x.joinable()) x.join();
    done_ = true;
  }
  ~HostFill() { finish(nullptr, nullptr); }

 private:
  void run(int t) {
    const long long j0 = (long long)n_ * t / nt_, j1 = (long long)n_ * (t + 1) / nt_;
    if (ld_ == n_) {
      memset(z_ + j0 * n_, 0, (size_t)(j1 - j0) * n_ * sizeof(double));
    } else {
      for (long long j = j0; j < j1; ++j) memset(z_ + j * ld_, 0, (size_t)n_ * sizeof(double));
    }
    const PackedZ *pz;
    const double *src;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [this] { return ready_; });
      pz = pz_;
      src = src_;
    }
    if (!pz) return;
    for (long long j = j0; j < j1; ++j) {
      const int2 r = pz->seg[j];
      if (r.y > r.x)
        memcpy(z_ + j * ld_ + r.x, src + pz->off[j], (size_t)(r.y - r.x) * sizeof(double));
    }
  }
  double *z_;
  int n_;
  long long ld_;
  int nt_ = 0;
  std::vector<std::thread> th_;
  std::vector<int> inline_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool ready_ = false, on_ = false, done_ = false;
  const PackedZ *pz_ = nullptr;
  const double *src_ = nullptr;
};

}  // namespace hss
