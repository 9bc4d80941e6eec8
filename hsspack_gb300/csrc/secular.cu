// secular.cu -- secular equation, Loewner z-hat and eigenvector scalings on sm_103a.
//
// One warp solves one root of
//     f(x) = 1/rho + sum_i z_i^2 / (d_i - x) = 0 ,   d_0 < d_1 < ... < d_{K-1},
// (the DLAED4 calls of SRC/mdlaed3.f90:207-225).  The method is the "middle
// way" rational iteration of R.-C. Li (1993) as analysed by Gu & Eisenstat
// (1995): the sums left and right of the root are each replaced by a one-pole
// rational model matching value and slope at the current iterate, and the
// two-pole model equation is solved in closed form.  A bracket keeps every
// iterate inside the pole interval; a step that leaves it is replaced by
// bisection.  All arithmetic is FP64.  Lanes split the pole sums; the five
// partial sums are combined by butterfly shuffles, so every lane holds
// identical values and the scalar control flow is uniform across the warp.
//
// Positions are measured from the nearer pole ("origin") so that the gaps
// d_i - x near the root keep full relative accuracy; DIFL/DIFR are formed from
// those gaps exactly as LAPACK's DELTA output is used at mdlaed3.f90:215-216.
#include <atomic>

#include "hss_common.cuh"
#include "hss_kernels.h"

namespace hss {

struct SecSums {
  double psi, dpsi, phi, dphi, eabs;
};

// Sum over the L lanes of one root group (xor offsets < L stay in the group;
// every lane of the warp takes part, so the shuffles are never divergent).
template <int L>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(HSS_FULL, v, o);
  return v;
}

// Sums over i of z_i^2/(p_i - x) split at jl (psi: i <= jl, phi: i > jl),
// their derivatives, and sum |z_i^2/(p_i - x)| for the rounding-error bound.
// x = p_oi + tau; every gap is formed as (p_i - p_oi) - tau.  Poles p_i = d_i,
// or p_i = d_i^2 in singular-value mode (SQ, DLASD4's equation
// 1 + sum z_i^2 / (d_i^2 - sigma^2) = 0) with p_i - p_oi = (d_i - d_oi)(d_i + d_oi).
// Lane gl of the group takes terms gl, gl + L, ...
template <int L, bool SQ>
__device__ __forceinline__ SecSums sec_eval(const double *__restrict__ d,
                                            const double *__restrict__ z, int K, int oi,
                                            double tau, int jl, int gl) {
  // Every lane of the warp calls this (lanes without a root pass K = 0).
  // Each side of the split (i <= jl, i > jl) holds terms of one sign, so
  // sum |v| = |psi| + |phi|; and the stretches that are on the same side for
  // every lane of the warp (below the warp's smallest jl, above its largest)
  // are summed without a per-term branch.
  double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
  const double o = K > 0 ? __ldg(d + oi) : 0.0;
  const int jlo = __reduce_min_sync(HSS_FULL, K > 0 ? jl : (1 << 29));
  const int jhi = __reduce_max_sync(HSS_FULL, K > 0 ? jl : -1);
  // t = z_i / (d_i - x); the sums take z_i t and t^2 by fused multiply-adds
  auto term = [&](int i, double &zi, double &t) {
    zi = __ldg(z + i);
    const double di = __ldg(d + i);
    const double del = (SQ ? (di - o) * (di + o) : (di - o)) - tau;
    t = zi * rcp_nr(del);
  };
  int i = gl;
  for (const int e = min(K, jlo + 1); i < e; i += L) {
    double zi, t;
    term(i, zi, t);
    a0 = fma(zi, t, a0); a1 = fma(t, t, a1);
  }
  for (const int e = min(K, jhi + 1); i < e; i += L) {
    double zi, t;
    term(i, zi, t);
    if (i <= jl) { a0 = fma(zi, t, a0); a1 = fma(t, t, a1); }
    else { b0 = fma(zi, t, b0); b1 = fma(t, t, b1); }
  }
  for (; i < K; i += L) {
    double zi, t;
    term(i, zi, t);
    b0 = fma(zi, t, b0); b1 = fma(t, t, b1);
  }
  SecSums s;
  s.psi = group_sum<L>(a0); s.dpsi = group_sum<L>(a1);
  s.phi = group_sum<L>(b0); s.dphi = group_sum<L>(b1);
  s.eabs = fabs(s.psi) + fabs(s.phi);
  return s;
}

// Root of  c + A/(da - t) + B/(db - t) = 0  inside (lo, hi); returns false if
// neither root of the equivalent quadratic lies there.
__device__ __forceinline__ bool two_pole_root(double c, double A, double B, double da,
                                              double db, double lo, double hi,
                                              double &t) {
  const double a2 = c;
  const double a1 = -(c * (da + db) + A + B);
  const double a0 = c * da * db + A * db + B * da;
  double r1, r2;
  if (a2 == 0.0) {
    if (a1 == 0.0) return false;
    r1 = r2 = -a0 / a1;
  } else {
    double disc = a1 * a1 - 4.0 * a2 * a0;
    if (disc < 0.0) disc = 0.0;
    const double q = -0.5 * (a1 + copysign(sqrt(disc), a1));
    r1 = q / a2;
    r2 = (q != 0.0) ? a0 / q : r1;
  }
  const bool ok1 = r1 > lo && r1 < hi, ok2 = r2 > lo && r2 < hi;
  if (ok1 && ok2) {  // both inside: take the one nearer the bracket middle
    const double m = 0.5 * (lo + hi);
    t = fabs(r1 - m) <= fabs(r2 - m) ? r1 : r2;
    return true;
  }
  if (ok1) { t = r1; return true; }
  if (ok2) { t = r2; return true; }
  return false;
}

// Per-root iteration state.  A group of L lanes owns one root; all lanes of a
// group hold identical copies.  The warp loops until every group converged;
// finished groups keep taking part in the (harmless) shuffles.
struct RootState {
  const double *d, *z;
  int K, j, jl, jr, oi;  // oi: index of the origin pole
  bool sq;               // singular-value mode: poles d_i^2
  double rho, rhoinv, tau, lo, hi, delta, top;
  int phase;  // 0: first evaluation (midpoint), 1: iterating, 2: done
  int iters, status;
  bool last;
  bool learned;  // started from the learned position; checked at the first step
  bool fell_back;
  bool fw;       // step model: false middle way, true fixed weight (origin pole exact)
  double prew;   // residual of the previous step (0: none yet)
  double prel;   // previous model step / distance to the origin pole (< 0: none)
  int first;     // evaluation count at the first evaluation of a given start
};

__device__ __forceinline__ double pole(const RootState &r, int i) { return __ldg(r.d + i); }
// p_i - p_k, exactly as the pole sums form it
__device__ __forceinline__ double pdiff(const RootState &r, int i, int k) {
  const double a = pole(r, i), b = pole(r, k);
  return r.sq ? (a - b) * (a + b) : a - b;
}
// p_i - origin
__device__ __forceinline__ double gap(const RootState &r, int i) { return pdiff(r, i, r.oi); }

// First evaluation point: the midpoint of the pole interval (standard guess),
// or the learned position (phase 1 directly).
// guess: signed distance of the start to the nearer pole in units of the
// interval (|guess| <= 1/2; anything else: the standard midpoint start).
// full: the start's side is not known (an FP32 pre-solve) -- the bracket is
// the whole interval; otherwise (a learned start after the FP64 midpoint
// evaluation) the half interval.
__device__ __forceinline__ void root_init(RootState &r, float guess, double zsq, bool full,
                                          float4 ref = make_float4(0.f, 0.f, 0.f, 0.f)) {
  r.rhoinv = 1.0 / r.rho;
  r.iters = 0;
  r.status = HSS_OK;
  r.last = (r.j == r.K - 1);
  r.jl = r.last ? r.K - 2 : r.j;
  r.jr = r.jl + 1;
  r.delta = r.last ? 0.0 : pdiff(r, r.j + 1, r.j);
  r.top = r.rho * zsq;
  r.phase = 0;
  r.learned = false;
  r.fell_back = false;
  r.fw = false;
  r.prew = 0.0;
  r.prel = -1.0;
  r.first = 0;
  if (!r.last) {
    r.oi = r.j;
    r.tau = 0.5 * r.delta;
    if (guess != 0.0f && fabsf(guess) <= 0.5f) {  // learned signed distance to the nearer pole
      // the midpoint pass already fixed the half interval (one evaluation)
      const double half = full ? r.delta : 0.5 * r.delta;
      if (guess > 0.0f) { r.oi = r.j; r.tau = (double)guess * r.delta; r.lo = 0.0; r.hi = half; }
      else { r.oi = r.j + 1; r.tau = (double)guess * r.delta; r.lo = -half; r.hi = 0.0; }
      if (ref.x != 0.0f) {
        // a refined pre-solve: the start tau = x + y exactly (origin as the
        // guess's sign), and z its last step / tau, which counts as the
        // previous step of the quadratic-convergence acceptance
        r.tau = (double)ref.x + (double)ref.y;
        r.prel = (double)ref.z;
      }
      r.phase = 1;
      r.learned = true;
      r.iters = full ? 0 : 1;  // the learned start spent one evaluation on the midpoint
      r.first = r.iters + 1;
    }
  } else {
    r.oi = r.K - 1;
    r.tau = 0.5 * r.top;
  }
}

// The step of one root runs on one lane but takes a whole warp's FP64 issue
// slots, so its divides go through qdiv; a zero denominator gives NaN, which
// fails every bracket test below and falls back to bisection.
// Consume one evaluation at (o, tau).
__device__ __forceinline__ void root_step(RootState &r, const SecSums &s) {
  if (r.phase == 2) return;
  ++r.iters;
  const double zl = __ldg(r.z + r.jl), zr = __ldg(r.z + r.jr);
  const double w = r.rhoinv + s.psi + s.phi;
  if (r.phase == 0) {
    // two-pole model with the far poles frozen at the midpoint value
    const double gl = gap(r, r.jl) - r.tau, gr = gap(r, r.jr) - r.tau;
    const double c = w - zl * (zl / gl) - zr * (zr / gr);
    double t;
    if (!r.last) {
      const double tm = r.tau;
      if (w >= 0.0) {  // root in (d_j, midpoint]
        r.lo = 0.0; r.hi = tm;
        if (!two_pole_root(c, zl * zl, zr * zr, 0.0, r.delta, r.lo, r.hi, t)) t = 0.5 * tm;
      } else {         // root in (midpoint, d_{j+1}): measure from d_{j+1}
        r.oi = r.j + 1;
        r.lo = tm - r.delta; r.hi = 0.0;
        if (!two_pole_root(c, zl * zl, zr * zr, -r.delta, 0.0, r.lo, r.hi, t)) t = 0.5 * r.lo;
      }
    } else {
      const double tm = r.tau;
      const double da = gap(r, r.jl);
      if (w >= 0.0) { r.lo = 0.0; r.hi = tm; }
      else { r.lo = tm; r.hi = r.top * (1.0 + 4.0 * HSS_EPS); }
      if (!two_pole_root(c, zl * zl, zr * zr, da, 0.0, r.lo, r.hi, t)) t = 0.5 * (r.lo + r.hi);
    }
    r.tau = t;
    r.phase = 1;
    return;
  }
  // middle-way step
  const double dw = s.dpsi + s.dphi;
  if (!(fabs(w) <= 1.7e308) || !(dw <= 1.7e308)) {  // overflow next to a pole: bisect
    if (r.iters > 41) { r.status = HSS_SECULAR_NOCONV; r.phase = 2; return; }
    r.learned = false;
    r.tau = 0.5 * (r.lo + r.hi);
    return;
  }
  const double erretm = 8.0 * s.eabs + 2.0 * r.rhoinv + 3.0 * fabs(r.tau) * dw;
  if (fabs(w) <= HSS_EPS * erretm) { r.phase = 2; return; }
  if (r.iters > 41) { r.status = HSS_SECULAR_NOCONV; r.phase = 2; return; }
  if (r.learned && r.iters == r.first) {
    // residual check of the learned start: a Newton step across most of the
    // half interval means the start is unusable; restart from the standard guess
    r.learned = false;
    if (!(fabs(w / dw) <= 0.45 * r.delta)) {
      r.fell_back = true;
      r.prew = 0.0;
      r.prel = -1.0;
      r.phase = 0;
      r.oi = r.j;
      r.tau = 0.5 * r.delta;
      return;
    }
  }
  // a residual that kept its sign and fell by less than 10x: change the model
  if (!r.last && w * r.prew > 0.0 && fabs(w) > 0.1 * fabs(r.prew)) r.fw = !r.fw;
  r.prew = w;
  if (w < 0.0) r.lo = fmax(r.lo, r.tau); else r.hi = fmin(r.hi, r.tau);
  // Two-pole model  c + s_l/(gl - eta) + s_r/(gr - eta)  matching w and dw at
  // eta = 0; cleared of denominators it is  c eta^2 - a eta + b = 0, and only
  // c depends on how dw is shared between the two poles.
  const double gl = gap(r, r.jl) - r.tau;
  const double gr = gap(r, r.jr) - r.tau;
  const double a = (gl + gr) * w - gl * gr * dw;
  const double b = gl * gr * w;
  double c;
  if (!r.fw) {  // middle way: each side's sum on its own pole
    c = w - gl * s.dpsi - gr * s.dphi;
  } else if (r.oi == r.j) {  // fixed weight: origin pole exact, the rest on the other
    const double t = qdiv(__ldg(r.z + r.jl), gl), q = t * t;
    c = w - gr * dw - (gl - gr) * q;
  } else {
    const double t = qdiv(__ldg(r.z + r.jr), gr), q = t * t;
    c = w - gl * dw - (gr - gl) * q;
  }
  double eta;
  if (r.last) {
    // the root lies beyond both poles (gl, gr < 0): the larger root of the
    // quadratic; c < 0 only from rounding
    c = fabs(c);
    if (c == 0.0) {
      eta = r.hi - r.tau;  // no root beyond the poles: bisect
    } else {
      double disc = a * a - 4.0 * b * c;
      if (disc < 0.0) disc = 0.0;
      eta = (a >= 0.0) ? qdiv(a + sqrt(disc), 2.0 * c) : qdiv(2.0 * b, a - sqrt(disc));
    }
  } else if (c == 0.0) {
    eta = (a != 0.0) ? qdiv(b, a) : -qdiv(w, dw);
  } else {  // the root between the two poles
    double disc = a * a - 4.0 * b * c;
    if (disc < 0.0) disc = 0.0;
    eta = (a <= 0.0) ? qdiv(a - sqrt(disc), 2.0 * c) : qdiv(2.0 * b, a + sqrt(disc));
  }
  if (w * eta >= 0.0) eta = -qdiv(w, dw);  // model went the wrong way: Newton step
  double tn = r.tau + eta;
  const bool bisect = !(tn > r.lo && tn < r.hi);
  if (bisect) {
    // bisect; geometrically when the bracket spans decades on one side of the
    // origin (roots next to a pole sit many decades below the interval)
    if (r.lo > 0.0 && r.hi > 4096.0 * r.lo) tn = sqrt(r.lo * r.hi);
    else if (r.hi < 0.0 && r.lo < 4096.0 * r.hi) tn = -sqrt(r.lo * r.hi);
    else tn = 0.5 * (r.lo + r.hi);
  }
  const double step = tn - r.tau;
  r.tau = tn;
  if (!r.last) {  // keep the origin at the pole nearer the iterate
    if (r.oi == r.j && r.tau > 0.5 * r.delta) {
      r.oi = r.j + 1; r.tau -= r.delta; r.lo -= r.delta; r.hi -= r.delta;
    } else if (r.oi == r.j + 1 && r.tau < -0.5 * r.delta) {
      r.oi = r.j; r.tau += r.delta; r.lo += r.delta; r.hi += r.delta;
    }
  }
  if (fabs(step) <= 2.0 * HSS_EPS * fabs(r.tau) || r.hi - r.lo <= 2.0 * HSS_EPS * fabs(r.tau)) {
    r.phase = 2;
    return;
  }
  // Quadratic convergence seen (a model step of at most 1e-10 of the
  // distance to the origin pole, and at most 100 x the square of the
  // previous relative step): the new iterate's error is below 1e-18 of that
  // distance, so it is final without another evaluation.
  const double rel = qdiv(fabs(step), fmax(fabs(r.tau), 1e-300));
  if (!bisect && r.prel >= 0.0 && rel <= 1e-10 && rel <= 100.0 * r.prel * r.prel) {
    r.phase = 2;
    return;
  }
  r.prel = bisect ? -1.0 : rel;
}

// Outputs of one finished root (lam, DIFL, DIFR, iteration counts, status);
// K = 1 is solved here in closed form.
template <bool SQ>
__device__ __forceinline__ void secular_out(RootState &st, int s, double *__restrict__ lam,
                                            double *__restrict__ difl, double *__restrict__ difr,
                                            int *__restrict__ iters, int *__restrict__ status,
                                            unsigned long long *__restrict__ itsum) {
  double lm, dfl, dfr;
  if (st.K == 1) {
    const double zz = __ldg(st.z) * __ldg(st.z);
    const double d0 = __ldg(st.d);
    if (SQ) {  // sigma^2 = d_0^2 + rho z^2
      lm = d0 + st.rho * zz / (d0 + sqrt(d0 * d0 + st.rho * zz));
      dfl = lm - d0;
    } else {
      lm = d0 + st.rho * zz; dfl = st.rho * zz;
    }
    dfr = 0.0;
    st.iters = 0; st.status = HSS_OK; st.fell_back = false;
  } else if (SQ) {
    // sigma = sqrt(d_o^2 + tau) = d_o + tau / (d_o + sigma); DIFL / DIFR as
    // sigma - d from (sigma^2 - d^2) / (sigma + d)
    const double o = pole(st, st.oi);
    lm = o + st.tau / (o + sqrt(o * o + st.tau));
    dfl = (st.tau - gap(st, st.j)) / (lm + pole(st, st.j));
    dfr = st.last ? 0.0 : (st.tau - gap(st, st.j + 1)) / (lm + pole(st, st.j + 1));
  } else {
    lm = pole(st, st.oi) + st.tau;
    dfl = -(gap(st, st.j) - st.tau);
    dfr = st.last ? 0.0 : -(gap(st, st.j + 1) - st.tau);
  }
  lam[s + st.j] = lm;
  difl[s + st.j] = dfl;
  difr[s + st.j] = dfr;
  if (iters) iters[s + st.j] = st.iters;
  if (itsum) {
    atomicAdd(itsum, (unsigned long long)st.iters);
    if (st.fell_back) atomicAdd(itsum + 1, 1ull);
    atomicAdd(itsum + 2, (unsigned long long)st.iters * (unsigned long long)st.K);  // pole terms
  }
  if (st.status) atomicMax(status, st.status);
}

// One lane per root with a sequence of roots per lane (wide levels): lane l of
// the T launched takes roots l, l + T, l + 2T, ..., starting the next as soon as
// its current one has converged.  A warp then costs the largest per-lane sum
// of evaluations instead of, root after root, the largest evaluation count of
// its 32 roots (the FP64 pipe is charged per warp instruction, idle lanes
// included).
template <bool SQ>
__device__ __forceinline__ void secular_lanes(const LevelView &lv, const double *__restrict__ dl,
                                              const double *__restrict__ zw,
                                              double *__restrict__ lam, double *__restrict__ difl,
                                              double *__restrict__ difr, int *__restrict__ iters,
                                              int *__restrict__ status,
                                              unsigned long long *__restrict__ itsum,
                                              const float *__restrict__ guess, bool full,
                                              const float4 *__restrict__ gref) {
  const int total = __ldg(lv.rootoff + lv.P);
  const long long T = (long long)gridDim.x * blockDim.x;
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  RootState st;
  st.K = 0; st.j = 0; st.jl = 0; st.oi = 0; st.tau = 0.0; st.phase = 2;
  st.d = dl; st.z = zw;
  int s = 0;
  bool act = false;
  auto next = [&]() {  // the lane's next root that needs the iteration
    act = false;
    for (; r < total; r += T) {
      const int m = find_merge(lv.rootoff, lv.P, (int)r);
      s = __ldg(lv.s + m);
      st.j = (int)r - __ldg(lv.rootoff + m);
      st.K = __ldg(lv.K + m);
      st.rho = __ldg(lv.rho + m);
      st.d = dl + s;
      st.z = zw + s;
      st.sq = SQ;
      st.oi = 0;
      if (st.K == 1) {
        secular_out<SQ>(st, s, lam, difl, difr, iters, status, itsum);
        continue;
      }
      double zsq = 0.0;  // the last root's bound only
      if (st.j == st.K - 1)
        for (int i = 0; i < st.K; ++i) zsq += __ldg(st.z + i) * __ldg(st.z + i);
      root_init(st, guess ? __ldg(guess + s + st.j) : 2.0f, zsq, full,
                gref ? gref[s + st.j] : make_float4(0.f, 0.f, 0.f, 0.f));
      act = true;
      return;
    }
  };
  next();
  while (__any_sync(HSS_FULL, act)) {
    const SecSums sm = sec_eval<1, SQ>(st.d, st.z, act ? st.K : 0, st.oi, st.tau, st.jl, 0);
    if (act) {
      root_step(st, sm);
      if (st.phase == 2) {
        secular_out<SQ>(st, s, lam, difl, difr, iters, status, itsum);
        r += T;
        next();
      }
    }
  }
}

// ------------------------------------------------------------- kernels -----
// Batched over the merges of one DC level (find_merge: hss_common.cuh).

// One root per group of L lanes (L = 1..32 chosen from the level's largest
// K so that each lane sums ~8 pole terms and the group reductions stay cheap).
template <int L, bool SQ>
__global__ void __launch_bounds__(256)
k_secular(LevelView lv, const double *__restrict__ dl, const double *__restrict__ zw,
          double *__restrict__ lam, double *__restrict__ difl, double *__restrict__ difr,
          int *__restrict__ iters, int *__restrict__ status, unsigned long long *__restrict__ itsum,
          const float *__restrict__ guess, bool full, const float4 *__restrict__ gref,
          bool lanes) {
  if (L == 1 && lanes) {
    secular_lanes<SQ>(lv, dl, zw, lam, difl, difr, iters, status, itsum, guess, full, gref);
    return;
  }
  const int lane = threadIdx.x & 31, gl = lane & (L - 1);
  const int r = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) / L);
  const int total = __ldg(lv.rootoff + lv.P);
  RootState st;
  int s = 0;
  const bool valid = r < total;
  if (valid) {
    const int m = find_merge(lv.rootoff, lv.P, r);
    s = __ldg(lv.s + m);
    st.j = r - __ldg(lv.rootoff + m);
    st.K = __ldg(lv.K + m);
    st.rho = __ldg(lv.rho + m);
  } else {
    st.j = 0; st.K = 0; st.rho = 1.0;
  }
  st.d = dl + s;
  st.z = zw + s;
  st.sq = SQ;
  st.oi = 0;
  // sum z^2 bounds the last root only (the root beyond every pole): the other
  // roots skip that pass over the poles (the group sum still runs on every lane)
  double zsq = 0.0;
  const int kz = (valid && st.j == st.K - 1) ? st.K : 0;
  for (int i = gl; i < kz; i += L) zsq += __ldg(st.z + i) * __ldg(st.z + i);
  zsq = group_sum<L>(zsq);
  const bool trivial = !valid || st.K == 1;
  if (!trivial)
    root_init(st, guess ? __ldg(guess + s + st.j) : 2.0f, zsq, full,
              gref ? gref[s + st.j] : make_float4(0.f, 0.f, 0.f, 0.f));
  else st.phase = 2;
  while (__any_sync(HSS_FULL, st.phase != 2)) {
    const SecSums sm = sec_eval<L, SQ>(st.d, st.z, st.phase == 2 ? 0 : st.K, st.oi, st.tau, st.jl,
                                       gl);
    // the scalar step runs on the group's first lane only (FP64 issue slots
    // are scarce on this part); the others receive what the next pole sums need
    if (L == 1 || gl == 0) root_step(st, sm);
    if (L > 1) {
      const int lead = lane & ~(L - 1);
      st.tau = __shfl_sync(HSS_FULL, st.tau, lead);
      st.oi = __shfl_sync(HSS_FULL, st.oi, lead);
      st.phase = __shfl_sync(HSS_FULL, st.phase, lead);
    }
  }
  if (valid && gl == 0) secular_out<SQ>(st, s, lam, difl, difr, iters, status, itsum);
}

// Loewner: z_hat_i^2 = prod_j (d_i - lam_j) / prod_{j != i} (d_i - d_j)
// (SRC/mdlaed3.f90:217-230).  Numerators and denominators are multiplied
// separately and renormalised by their binary exponents every 8 factors, so
// there is one multiply per factor and no division in the O(K^2) loop.
//   Singular-value mode (sq): z_hat_i^2 = prod_j (sigma_j^2 - d_i^2) /
// prod_{j != i} (d_j^2 - d_i^2) (the z recomputation of DLASD3 / MDLASD8), every
// factor formed as a product of a difference and a sum.
template <int L>
__global__ void k_lowner(LevelView lv, const double *__restrict__ dl,
                         const double *__restrict__ difl, const double *__restrict__ difr,
                         const double *__restrict__ zw, double *__restrict__ zhat, bool sq) {
  // one root per group of L lanes (as the secular kernel); every lane of the
  // warp takes part in the group shuffles
  const int lane = threadIdx.x & 31, gl = lane & (L - 1);
  const int r = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) / L);
  const bool valid = r < __ldg(lv.rootoff + lv.P);
  int i = 0, s = 0, K = 0;
  if (valid) {
    const int m = find_merge(lv.rootoff, lv.P, r);
    i = r - __ldg(lv.rootoff + m);
    s = __ldg(lv.s + m);
    K = __ldg(lv.K + m);
  }
  PoleDiff P{dl + s, difl + s, difr + s, sq};
  const double di = valid ? __ldg(dl + s + i) : 0.0;
  double num = 1.0, den = 1.0;
  int en = 0, ed = 0, cnt = 0;
  for (int j = gl; j < K; j += L) {
    num *= P.fd(i, j);
    if (j != i) {
      const double dj = __ldg(dl + s + j);
      den *= sq ? (di - dj) * (di + dj) : (di - dj);
    }
    if (++cnt == 8) {
      int e;
      num = frexp(num, &e); en += e;
      den = frexp(den, &e); ed += e;
      cnt = 0;
    }
  }
  {
    int e;
    num = frexp(num, &e); en += e;
    den = frexp(den, &e); ed += e;
  }
#pragma unroll
  for (int ofs = L / 2; ofs > 0; ofs >>= 1) {
    double on = __shfl_xor_sync(HSS_FULL, num, ofs);
    double od = __shfl_xor_sync(HSS_FULL, den, ofs);
    int oen = __shfl_xor_sync(HSS_FULL, en, ofs);
    int oed = __shfl_xor_sync(HSS_FULL, ed, ofs);
    int e;
    num = frexp(num * on, &e); en += oen + e;
    den = frexp(den * od, &e); ed += oed + e;
  }
  if (valid && gl == 0) {
    const double q = ldexp(fabs(num / den), en - ed);
    zhat[s + i] = copysign(sqrt(q), __ldg(zw + s + i));
  }
}

// alpha_j = 1 / || (z_hat_i / (d_i - lam_j))_i ||_2  (SRC/mdlaed3.f90:233-249).
__global__ void k_alpha(LevelView lv, const double *__restrict__ dl,
                        const double *__restrict__ difl, const double *__restrict__ difr,
                        const double *__restrict__ zhat, double *__restrict__ alpha, bool sq) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= __ldg(lv.rootoff + lv.P)) return;
  const int m = find_merge(lv.rootoff, lv.P, r);
  const int j = r - __ldg(lv.rootoff + m);
  const int s = __ldg(lv.s + m);
  const int K = __ldg(lv.K + m);
  PoleDiff P{dl + s, difl + s, difr + s, sq};
  double acc = 0.0;
  for (int i = lane; i < K; i += HSS_WARP) {
    const double w = __ldg(zhat + s + i) * rcp_nr(P.fd(i, j));
    acc += w * w;
  }
  acc = warp_sum(acc);
  if (lane == 0) alpha[s + j] = 1.0 / sqrt(acc);
}

// Dense eigenvector block of the rank-one update for the small-K merges
// (LAPACK DLAED3's S, used at SRC/mdlaed1.f90:198-201): column j holds
// z_hat_i / (d_i - lam_j) normalised to unit length.  Row i is written at
// group position grp[s+i] (columns of Q2 grouped by block structure) of a
// per-merge K x K column-major buffer starting at Sws + soff[m].
__global__ void k_build_S(LevelView lv, const double *__restrict__ dl,
                          const double *__restrict__ difl, const double *__restrict__ difr,
                          const double *__restrict__ zhat, const int *__restrict__ grp,
                          const long long *__restrict__ soff, double *__restrict__ Sws) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= __ldg(lv.rootoff + lv.P)) return;
  const int m = find_merge(lv.rootoff, lv.P, r);
  const int j = r - __ldg(lv.rootoff + m);
  const int s = __ldg(lv.s + m);
  const int K = __ldg(lv.K + m);
  double *S = Sws + __ldg(soff + m) + (long long)j * K;
  if (K == 1) {
    if (lane == 0) S[0] = 1.0;
    return;
  }
  PoleDiff P{dl + s, difl + s, difr + s};
  double acc = 0.0;
  for (int i = lane; i < K; i += HSS_WARP) {
    const double w = __ldg(zhat + s + i) * rcp_nr(P.fd(i, j));
    S[__ldg(grp + s + i)] = w;
    acc += w * w;
  }
  acc = warp_sum(acc);
  const double a = 1.0 / sqrt(acc);
  __syncwarp();
  for (int i = lane; i < K; i += HSS_WARP) {
    const int g = __ldg(grp + s + i);
    S[g] *= a;
  }
}

// Dense Cauchy-like block for the standalone API.
__global__ void k_cauchy_eig(int K, const double *__restrict__ F, const double *__restrict__ u,
                             const double *__restrict__ v, const double *__restrict__ difl,
                             const double *__restrict__ difr, double *__restrict__ C, bool sq) {
  PoleDiff P{F, difl, difr, sq};
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)K * K) return;
  const int i = (int)(idx % K), j = (int)(idx / K);
  C[idx] = __ldg(u + i) * __ldg(v + j) / P.fd(i, j);
}

__global__ void k_cauchylike(int M, int N, const double *__restrict__ D,
                             const double *__restrict__ F, const double *__restrict__ u,
                             const double *__restrict__ v, double *__restrict__ A) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)M * N) return;
  const int i = (int)(idx % M), j = (int)(idx / M);
  A[idx] = __ldg(u + i) * __ldg(v + j) / (__ldg(D + i) - __ldg(F + j));
}

// Midpoint pass for the learned start: per non-last root, the full secular
// sums at the midpoint of (d_j, d_{j+1}) (the standard method's first
// evaluation) turned into the predictor's features (see predictor.cu).
// Root of the two-pole model  c - a/t + b/(1-t) = 0  in (0, 1), returned as
// the distance u to the nearer pole (side 0: t = u, side 1: t = 1 - u), each
// side solved from its own quadratic so that u keeps full relative accuracy.
__device__ __forceinline__ double small_root(double A, double B, double C) {
  // root of A u^2 + B u + C = 0 nearest 0 (stable form)
  if (fabs(A) < 1e-300) return -C / B;
  double disc = B * B - 4.0 * A * C;
  disc = disc < 0.0 ? 0.0 : disc;
  const double q = -0.5 * (B + copysign(sqrt(disc), B));
  return (q != 0.0) ? C / q : -B / (2.0 * A);
}
__device__ __forceinline__ double pole_root_u(double c, double a, double b, int &side) {
  // side 0:  c t(1-t) - a(1-t) + b t = 0   ->  -c t^2 + (c+a+b) t - a = 0
  // side 1 (t = 1-u):  -c u^2 + (c-a-b) u + b = 0
  const double f_half = c - 2.0 * a + 2.0 * b;  // delta*f at t = 1/2
  double u;
  if (f_half >= 0.0) { side = 0; u = small_root(-c, c + a + b, -a); }
  else { side = 1; u = small_root(-c, c - a - b, b); }
  if (!(u > 0.0)) u = 1e-300;
  return fmin(u, 0.5);
}
__device__ __forceinline__ double logit_u(double u, int side) {
  const double l = log(u / (1.0 - u));
  return side == 0 ? l : -l;
}

// FP32 copies of a level's poles and weights (for the FP32 pre-solve).
__global__ void k_to_f32(int n, const double *__restrict__ a, const double *__restrict__ b,
                         float *__restrict__ fa, float *__restrict__ fb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { fa[i] = (float)a[i]; fb[i] = (float)b[i]; }
}

// Float-float arithmetic (value = hi + lo, |lo| <= ulp(hi) / 2; Dekker 1971,
// Knuth's TwoSum): about 48 significant bits from FP32 instructions.
__device__ __forceinline__ void ff_two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void ff_add(float ah, float al, float bh, float bl, float &sh,
                                       float &sl) {
  float s1, e1;
  ff_two_sum(ah, bh, s1, e1);
  e1 += al + bl;
  sh = s1 + e1;
  sl = e1 - (sh - s1);
}
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float &ph,
                                       float &pl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);  // the exact error of the product
  e += ah * bl + al * bh;
  ph = p + e;
  pl = e - (ph - p);
}
__device__ __forceinline__ void ff_div(float ah, float al, float bh, float bl, float &qh,
                                       float &ql) {
  const float q1 = ah / bh;
  const float p = q1 * bh, pe = fmaf(q1, bh, -p);
  const float r = (((ah - p) - pe) + al) - q1 * bl;  // a - q1 b
  const float q2 = r / bh;
  qh = q1 + q2;
  ql = q2 - (qh - q1);
}

// FP32 copies plus the float-float splits the refined pre-solve needs: poles
// d = dh + dl, and z^2 = z2h + z2l (z^2 formed in FP64), once per level.
__global__ void k_to_ff(int n, const double *__restrict__ a, const double *__restrict__ b,
                        float *__restrict__ fa, float *__restrict__ fb, float *__restrict__ fal,
                        float *__restrict__ z2h, float *__restrict__ z2l) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = a[i], z = b[i], z2 = z * z;
  const float dh = (float)d, zh2 = (float)z2;
  fa[i] = dh;
  fal[i] = (float)(d - (double)dh);
  fb[i] = (float)z;
  z2h[i] = zh2;
  z2l[i] = (float)(z2 - (double)zh2);
}

template <int L>
__device__ __forceinline__ float group_sum_f(float v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(HSS_FULL, v, o);
  return v;
}

// Starting points of the FP64 iteration from a few steps of the same
// middle-way iteration in FP32 (this part issues FP32 instructions about sixty
// times faster than FP64 ones): gaps to the 2 GR nearest poles from FP64
// differences, the others from FP32 copies; start at the midpoint of
// (d_j, d_{j+1}), origin kept at the nearer pole, bracket safeguarding, at
// most 10 evaluations or until a step is below 4e-6 of the distance to the
// origin pole.  The result (a few 1e-6 of the interval at
// best) only starts the FP64 iteration, which decides convergence as before;
// guess[s + j] = signed distance to the nearer pole / interval, 0 for none.
// SQ: singular-value mode, the variable tau = sigma^2 - d_o^2 and the pole gaps
// (d_i - d_o)(d_i + d_o), as the FP64 kernel's squared mode.
// FF (refined pre-solve): after the FP32 iteration has converged, one more
// evaluation of the secular function in float-float arithmetic (every term, from
// the splits d32 + d32lo and z2h + z2l: no FP64 instruction per term) and one
// step from it; gref[s + j] = (tau, step, |step / tau|, 0), 0 when not refined.
// The FP64 iteration then starts at tau + step exactly, usually accepting after
// one evaluation (its first step shows quadratic convergence).
template <int L, bool SQ, bool FF>
__global__ void __launch_bounds__(256)
k_secular_guess32(LevelView lv, const double *__restrict__ dl, const float *__restrict__ d32,
                  const float *__restrict__ z32, float *__restrict__ guess,
                  const float *__restrict__ d32lo, const float *__restrict__ z2h,
                  const float *__restrict__ z2l, float4 *__restrict__ gref) {
  constexpr int GR = 4;
  const int lane = threadIdx.x & 31, gl = lane & (L - 1);
  const int r = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) / L);
  const int total = __ldg(lv.rootoff + lv.P);
  int s = 0, j = 0, K = 0;
  float rhoinv = 1.f;
  double rhoinv_d = 1.0;
  if (r < total) {
    const int m = find_merge(lv.rootoff, lv.P, r);
    s = __ldg(lv.s + m);
    j = r - __ldg(lv.rootoff + m);
    K = __ldg(lv.K + m);
    rhoinv_d = 1.0 / __ldg(lv.rho + m);
    rhoinv = (float)rhoinv_d;
  }
  const bool active = r < total && K >= 2 && j < K - 1;
  const int n0 = j - GR + 1;  // first near pole
  // near gaps d_i - d_o from FP64 differences, for the origin o = j or j + 1
  float gn[2 * GR];
  auto near_gaps = [&](int o) {
    const double dorg = active ? __ldg(dl + s + o) : 0.0;
#pragma unroll
    for (int q = 0; q < 2 * GR; ++q) {
      const int i = n0 + q;
      if (active && i >= 0 && i < K) {
        const double di = __ldg(dl + s + i);
        gn[q] = SQ ? (float)((di - dorg) * (di + dorg)) : (float)(di - dorg);
      } else {
        gn[q] = 0.f;
      }
    }
  };
  near_gaps(j);
  const float delta = gn[GR];  // d_{j+1} - d_j
  int o = j;
  float do32 = active ? __ldg(d32 + s + j) : 0.f;
  const int Ka = active ? K : 0;
  float tau = 0.5f * delta, lo = 0.f, hi = delta;
  bool done = !active, conv32 = false;
#pragma unroll 1
  for (int it = 0; it < 10; ++it) {
    float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
    if (!done) {
      for (int i = gl; i < Ka; i += L) {
        if (i >= n0 && i < n0 + 2 * GR) continue;  // the near poles follow
        const float zi = __ldg(z32 + s + i);
        const float di = __ldg(d32 + s + i);
        const float gi = SQ ? (di - do32) * (di + do32) : di - do32;
        const float t = __fdividef(zi, gi - tau);
        if (i <= j) { a0 = fmaf(zi, t, a0); a1 = fmaf(t, t, a1); }
        else { b0 = fmaf(zi, t, b0); b1 = fmaf(t, t, b1); }
      }
#pragma unroll
      for (int q = 0; q < 2 * GR; ++q) {
        const int i = n0 + q;
        if (i < 0 || i >= Ka || (i & (L - 1)) != gl) continue;
        const float zi = __ldg(z32 + s + i);
        const float t = __fdividef(zi, gn[q] - tau);
        if (i <= j) { a0 = fmaf(zi, t, a0); a1 = fmaf(t, t, a1); }
        else { b0 = fmaf(zi, t, b0); b1 = fmaf(t, t, b1); }
      }
    }
    a0 = group_sum_f<L>(a0); a1 = group_sum_f<L>(a1);
    b0 = group_sum_f<L>(b0); b1 = group_sum_f<L>(b1);
    if (!done) {
      const float w = rhoinv + a0 + b0, dw = a1 + b1;
      if (w == 0.f) {
        done = true;
      } else {
        if (w < 0.f) lo = fmaxf(lo, tau); else hi = fminf(hi, tau);
        const float gL = gn[GR - 1] - tau, gR = gn[GR] - tau;  // the poles j, j + 1
        const float A = (gL + gR) * w - gL * gR * dw;
        const float B = gL * gR * w;
        const float C = w - gL * a1 - gR * b1;
        float eta;
        if (C == 0.f) {
          eta = A != 0.f ? B / A : -w / dw;
        } else {
          const float disc = fmaxf(A * A - 4.f * B * C, 0.f);
          eta = A <= 0.f ? (A - sqrtf(disc)) / (2.f * C) : (2.f * B) / (A + sqrtf(disc));
        }
        if (!(w * eta < 0.f)) eta = -w / dw;  // wrong direction or not finite: Newton
        if (fabsf(eta) <= 4e-6f * fabsf(tau)) {  // FP32 resolution reached
          tau += eta;
          done = true;
          conv32 = true;
        } else {
          float tn = tau + eta;
          if (!(tn > lo && tn < hi)) tn = 0.5f * (lo + hi);
          tau = tn;
          // keep the origin at the pole nearer the iterate
          if (o == j && tau > 0.5f * delta) {
            o = j + 1; near_gaps(o); do32 = __ldg(d32 + s + o);
            tau -= delta; lo -= delta; hi -= delta;
          } else if (o == j + 1 && tau < -0.5f * delta) {
            o = j; near_gaps(o); do32 = __ldg(d32 + s + o);
            tau += delta; lo += delta; hi += delta;
          }
        }
      }
    }
  }
  float4 rf = make_float4(0.f, 0.f, 0.f, 0.f);
  if (FF) {
    const bool go = active && conv32 && tau != 0.f;
    float wh = 0.f, wl = 0.f, a1 = 0.f, b1 = 0.f;
    if (go) {
      const float dho = __ldg(d32 + s + o), dlo = __ldg(d32lo + s + o);
      for (int i = gl; i < Ka; i += L) {
        const float dhi = __ldg(d32 + s + i), dli = __ldg(d32lo + s + i);
        float gh, glo;  // d_i - d_o (squared mode: (d_i - d_o)(d_i + d_o))
        ff_add(dhi, dli, -dho, -dlo, gh, glo);
        if (SQ) {
          float ph, pl;
          ff_add(dhi, dli, dho, dlo, ph, pl);
          ff_mul(gh, glo, ph, pl, gh, glo);
        }
        float eh, el;  // gap - tau
        ff_add(gh, glo, -tau, 0.f, eh, el);
        float th, tl;
        ff_div(__ldg(z2h + s + i), __ldg(z2l + s + i), eh, el, th, tl);
        ff_add(wh, wl, th, tl, wh, wl);
        const float t = __fdividef(__ldg(z32 + s + i), eh);
        if (i <= j) a1 = fmaf(t, t, a1); else b1 = fmaf(t, t, b1);
      }
    }
#pragma unroll
    for (int q = L / 2; q > 0; q >>= 1) {  // group sums (every lane ends with the same bits)
      const float oh = __shfl_xor_sync(HSS_FULL, wh, q), ol = __shfl_xor_sync(HSS_FULL, wl, q);
      ff_add(wh, wl, oh, ol, wh, wl);
    }
    a1 = group_sum_f<L>(a1);
    b1 = group_sum_f<L>(b1);
    if (go) {
      const float rh = (float)rhoinv_d, rl = (float)(rhoinv_d - (double)rh);
      ff_add(wh, wl, rh, rl, wh, wl);
      const float w = wh, dw = a1 + b1;
      const float gL = gn[GR - 1] - tau, gR = gn[GR] - tau;  // the poles j, j + 1
      const float A = (gL + gR) * w - gL * gR * dw;
      const float B = gL * gR * w;
      const float C = w - gL * a1 - gR * b1;
      float eta;
      if (C == 0.f) {
        eta = A != 0.f ? B / A : -w / dw;
      } else {
        const float disc = fmaxf(A * A - 4.f * B * C, 0.f);
        eta = A <= 0.f ? (A - sqrtf(disc)) / (2.f * C) : (2.f * B) / (A + sqrtf(disc));
      }
      if (!(w * eta < 0.f)) eta = -w / dw;
      // only a correction well inside FP32's resolution is used
      if (fabsf(eta) <= 1e-4f * fabsf(tau)) rf = make_float4(tau, eta, fabsf(eta / tau), 0.f);
    }
  }
  if (r < total && gl == 0) {
    float g = 0.f;
    if (active) {
      g = tau / delta;  // from the origin pole: positive from d_j, negative from d_{j+1}
      if (g > 0.5f) { g -= 1.f; rf.x = 0.f; }
      else if (g < -0.5f) { g += 1.f; rf.x = 0.f; }
      if (!(fabsf(g) > 0.f && fabsf(g) <= 0.5f)) { g = 0.f; rf.x = 0.f; }
    }
    guess[s + j] = g;
    if (FF) gref[s + j] = rf;
  }
}

template <int L>
__global__ void __launch_bounds__(256)
k_secular_mid(LevelView lv, const double *__restrict__ dl, const double *__restrict__ zw,
              float *__restrict__ feat) {
  constexpr int NFP = 9;  // 8 features + side
  const int lane = threadIdx.x & 31, gl = lane & (L - 1);
  const int r = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) / L);
  const int total = __ldg(lv.rootoff + lv.P);
  int s = 0, j = 0, K = 0;
  double rho = 1.0;
  if (r < total) {
    const int m = find_merge(lv.rootoff, lv.P, r);
    s = __ldg(lv.s + m);
    j = r - __ldg(lv.rootoff + m);
    K = __ldg(lv.K + m);
    rho = __ldg(lv.rho + m);
  }
  const bool active = (r < total) && (j < K - 1) && K >= 2;
  const double *d = dl + s, *z = zw + s;
  double o = 0.0, tm = 0.0, delta = 1.0;
  if (active) {
    o = __ldg(d + j);
    delta = __ldg(d + j + 1) - o;
    tm = 0.5 * delta;
  }
  const SecSums sm = sec_eval<L, false>(d, z, active ? K : 0, j, tm, j, gl);
  if (r >= total || gl != 0) return;
  float *f = feat + (long long)(s + j) * NFP;
  if (!active) { f[NFP - 1] = -1.f; return; }
  const double zj = __ldg(z + j), zj1 = __ldg(z + j + 1);
  const double gl_ = (__ldg(d + j) - o) - tm, gr_ = (__ldg(d + j + 1) - o) - tm;
  const double w = 1.0 / rho + sm.psi + sm.phi, dw = sm.dpsi + sm.dphi;
  const double a = zj * zj, b = zj1 * zj1;
  const double c0 = delta * (w - zj * (zj / gl_) - zj1 * (zj1 / gr_));
  const double c1 = delta * delta * (dw - (zj / gl_) * (zj / gl_) - (zj1 / gr_) * (zj1 / gr_));
  int s0, s1;
  const double u0 = pole_root_u(c0, a, b, s0);
  const double t0 = s0 == 0 ? u0 : 1.0 - u0;
  const double u1 = pole_root_u(c0 + c1 * (t0 - 0.5), a, b, s1);
  const double ac = fmax(fabs(c0), 1e-300);
  const double gapl = (j > 0) ? (__ldg(d + j) - __ldg(d + j - 1)) / delta : 1e3;
  const double gapr = (j + 2 < K) ? (__ldg(d + j + 2) - __ldg(d + j + 1)) / delta : 1e3;
  auto cl = [](double x, double lo, double hi) { return (float)fmin(fmax(x, lo), hi); };
  f[0] = cl(log(a / ac + 1e-300), -60, 60);
  f[1] = cl(log(b / ac + 1e-300), -60, 60);
  f[2] = cl(c1 / ac, -1e3, 1e3);
  f[3] = c0 >= 0.0 ? 1.f : -1.f;
  f[4] = cl(log(gapl), -40, 40);
  f[5] = cl(log(gapr), -40, 40);
  f[6] = cl(logit_u(u0, s0), -700, 700);
  f[7] = cl(logit_u(u1, s1), -700, 700);
  f[8] = (w >= 0.0) ? 0.f : 1.f;  // root left / right of the midpoint
}

// ---------------------------------------------------------------- launch --
// Threads per CTA for the root kernels: 256 when the level fills the GPU
// several times over, else 64 so that a small level still spreads over all
// 152 SMs (the kernels use no shared memory and no block barriers).
static inline int root_block(long long threads) { return threads >= 152LL * 256 * 2 ? 256 : 64; }

static inline int warp_grid(int total, int threads) {
  return (int)(((long long)total * 32 + threads - 1) / threads);
}
// Pole terms per lane the lane-group width aims at (hss_config.sec_terms), and
// the thread count a level should reach.  Written by hss_set_config under the
// library lock but read by entry points that hold only their own lock (the
// no-allocation Loewner entry), hence relaxed atomics.
static std::atomic<int> g_sec_terms{8};
void set_secular_terms(int t) { g_sec_terms.store(t > 0 ? t : 8, std::memory_order_relaxed); }
static std::atomic<long long> g_sec_threads{152LL * 256};
void set_secular_threads(int t) {
  g_sec_threads.store(t > 0 ? t : 152LL * 256, std::memory_order_relaxed);
}

// Lanes per root of a level with `total` roots and largest merge maxk: the
// fewest lanes that (a) keep a lane's share at or below 64 pole terms and
// (b) give at least sec_threads threads (enough warps to keep the FP64 pipes
// of every SM busy), but never more than needed for sec_terms terms per lane.
// A level with many roots runs one lane per root (no per-root reduction or
// replicated step work); a level with few roots spreads each root.
static int lanes_per_root(int total, int maxk) {
  const int terms = g_sec_terms.load(std::memory_order_relaxed);
  const long long want = g_sec_threads.load(std::memory_order_relaxed);
  int cap = 1;
  while (cap < 32 && cap * terms < maxk) cap *= 2;
  int L = 1;
  while (L < cap && (L * 64 < maxk || (long long)total * L < want)) L *= 2;
  return L;
}

void launch_secular(const LevelView &lv, int total, int maxk, const double *dl, const double *zw,
                    double *lam, double *difl, double *difr, int *iters, int *status,
                    unsigned long long *itsum, const float *guess, cudaStream_t st, bool sq,
                    bool full, const float4 *gref) {
  if (total <= 0) return;
  const int L = lanes_per_root(total, maxk);
  int tb = root_block((long long)total * L);
  unsigned grid = (unsigned)(((long long)total * L + tb - 1) / tb);
  // wide levels at one root per lane: 152 x 512 lanes, each with a sequence of
  // roots (secular_lanes), once there are at least two roots per lane
  constexpr long long SEC_LANES = 152LL * 512;
  const bool lanes = L == 1 && total >= 2 * SEC_LANES;
  if (lanes) { tb = 256; grid = (unsigned)(SEC_LANES / tb); }
  switch (L * 2 + (sq ? 1 : 0)) {
#define SEC_CASE(LL, SQ)                                                                     \
  case LL * 2 + SQ:                                                                          \
    k_secular<LL, SQ><<<grid, tb, 0, st>>>(lv, dl, zw, lam, difl, difr, iters, status,     \
                                            itsum, guess, full, gref, lanes);                \
    break;
    SEC_CASE(1, 0) SEC_CASE(2, 0) SEC_CASE(4, 0) SEC_CASE(8, 0) SEC_CASE(16, 0) SEC_CASE(32, 0)
    SEC_CASE(1, 1) SEC_CASE(2, 1) SEC_CASE(4, 1) SEC_CASE(8, 1) SEC_CASE(16, 1) SEC_CASE(32, 1)
#undef SEC_CASE
  }
}
void launch_secular_guess32(const LevelView &lv, int total, int maxk, int npos,
                            const double *dl, const double *zw, float *d32, float *z32,
                            float *guess, cudaStream_t st, bool sq, float *d32lo, float *z2h,
                            float *z2l, float4 *gref) {
  if (total <= 0) return;
  const bool ff = gref != nullptr;
  if (ff) k_to_ff<<<(npos + 255) / 256, 256, 0, st>>>(npos, dl, zw, d32, z32, d32lo, z2h, z2l);
  else k_to_f32<<<(npos + 255) / 256, 256, 0, st>>>(npos, dl, zw, d32, z32);
  const int L = lanes_per_root(total, maxk);
  const int tb = root_block((long long)total * L);
  const unsigned grid = (unsigned)(((long long)total * L + tb - 1) / tb);
  const int mode = (sq ? 1 : 0) + (ff ? 2 : 0);
  switch (L * 4 + mode) {
#define G32_CASE(LL, SQ, FF)                                                         \
  case LL * 4 + (SQ ? 1 : 0) + (FF ? 2 : 0):                                         \
    k_secular_guess32<LL, SQ, FF><<<grid, tb, 0, st>>>(lv, dl, d32, z32, guess, d32lo, \
                                                       z2h, z2l, gref);                \
    break;
#define G32_ALL(LL) G32_CASE(LL, false, false) G32_CASE(LL, true, false) \
                    G32_CASE(LL, false, true) G32_CASE(LL, true, true)
    G32_ALL(1) G32_ALL(2) G32_ALL(4) G32_ALL(8) G32_ALL(16) G32_ALL(32)
#undef G32_ALL
#undef G32_CASE
  }
}
void launch_secular_mid(const LevelView &lv, int total, int maxk, const double *dl,
                        const double *zw, float *feat, cudaStream_t st) {
  if (total <= 0) return;
  const int L = lanes_per_root(total, maxk);
  const int tb = root_block((long long)total * L);
  const unsigned grid = (unsigned)(((long long)total * L + tb - 1) / tb);
  switch (L) {
#define MID_CASE(LL) \
  case LL: k_secular_mid<LL><<<grid, tb, 0, st>>>(lv, dl, zw, feat); break;
    MID_CASE(1) MID_CASE(2) MID_CASE(4) MID_CASE(8) MID_CASE(16) MID_CASE(32)
#undef MID_CASE
  }
}

void launch_lowner(const LevelView &lv, int total, const double *dl, const double *difl,
                   const double *difr, const double *zw, double *zhat, cudaStream_t st, bool sq,
                   int maxk) {
  if (total <= 0) return;
  const int L = lanes_per_root(total, maxk);
  const int tb = root_block((long long)total * L);
  const unsigned grid = (unsigned)(((long long)total * L + tb - 1) / tb);
  switch (L) {
#define LOW_CASE(LL) \
  case LL: k_lowner<LL><<<grid, tb, 0, st>>>(lv, dl, difl, difr, zw, zhat, sq); break;
    LOW_CASE(1) LOW_CASE(2) LOW_CASE(4) LOW_CASE(8) LOW_CASE(16) LOW_CASE(32)
#undef LOW_CASE
  }
}
void launch_alpha(const LevelView &lv, int total, const double *dl, const double *difl,
                  const double *difr, const double *zhat, double *alpha, cudaStream_t st,
                  bool sq) {
  if (total <= 0) return;
  const int tb = root_block((long long)total * 32);
  k_alpha<<<warp_grid(total, tb), tb, 0, st>>>(lv, dl, difl, difr, zhat, alpha, sq);
}
void launch_build_S(const LevelView &lv, int total, const double *dl, const double *difl,
                    const double *difr, const double *zhat, const int *grp,
                    const long long *soff, double *Sws, cudaStream_t st) {
  if (total <= 0) return;
  const int tb = root_block((long long)total * 32);
  k_build_S<<<warp_grid(total, tb), tb, 0, st>>>(lv, dl, difl, difr, zhat, grp, soff, Sws);
}
void launch_cauchy_eig(int K, const double *F, const double *u, const double *v,
                       const double *difl, const double *difr, double *C, cudaStream_t st, bool sq) {
  const long long tot = (long long)K * K;
  if (tot <= 0) return;
  k_cauchy_eig<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(K, F, u, v, difl, difr, C, sq);
}
__global__ void k_rcp(int n, const double *__restrict__ x, double *__restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = rcp_nr(x[i]);
}
void launch_rcp(int n, const double *x, double *y, cudaStream_t st) {
  if (n > 0) k_rcp<<<(n + 255) / 256, 256, 0, st>>>(n, x, y);
}
void launch_cauchylike(int M, int N, const double *D, const double *F, const double *u,
                       const double *v, double *A, cudaStream_t st) {
  const long long tot = (long long)M * N;
  if (tot <= 0) return;
  k_cauchylike<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(M, N, D, F, u, v, A);
}

}  // namespace hss
