// driver.cu -- host side of the GB300 divide-and-conquer eigensolver and the
// C ABI (include/hsspack_gb300.h).
//
// MDSTEDC (SRC/mdstedc.f90:139-436): split at negligible off-diagonals, scale
// each block, run the DC tree, unscale, order.  MDLAED0 (SRC/mdlaed0.f90:
// 121-380): halving tree down to SMLSIZ, batched leaf eigensolves, then one
// pass per level over all merges of the level.  Per level the host reads back
// only the merge sizes K (one small copy), plans workspaces, and launches each
// stage once for every merge of the level (cfg.batched = 1) or once per merge
// (cfg.batched = 0, the "plain" mode).
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <condition_variable>
#include <thread>
#include <vector>

#include "../../include/hsspack_gb300.h"
#include "hss_common.cuh"
#include "hss_gemm.h"
#include "hss_chol.h"
#include "hss_hss.h"
#include "hss_kernels.h"
#include "hss_pool.h"
#include "host_util.h"

namespace hss {

// ------------------------------------------------------------ device pool --
struct Buf {
  void *p = nullptr;
  size_t cap = 0;
};

struct TimedRange {
  int stage;
  cudaEvent_t a, b;
  long long bytes;
  double flops;
};

struct Ctx {
  std::recursive_mutex mu;
  std::vector<cudaEvent_t> evpool;
  size_t evused = 0;
  std::vector<TimedRange> ranges;
  cudaEvent_t open_ev[HSS_NSTAGE] = {};
  hss_config cfg;
  hss_stats stats;
  std::string err;
  std::map<std::string, Buf> bufs;
  bool pred_ready = false;  // learned secular predictor installed
  void *pinned = nullptr;
  size_t pinned_cap = 0;
  char *ring = nullptr;  // pinned staging ring for parameter uploads
  size_t ring_cap = 0, ring_head = 0;
  struct RingUse {  // ring bytes [a, b) are read by copies before event ev
    size_t a, b;
    cudaEvent_t ev;
  };
  std::deque<RingUse> ring_uses;     // in allocation order
  std::vector<cudaEvent_t> ring_ev;  // free events
  PackedZ *pz = nullptr;             // packed-output request of the running solve
  double *zstage = nullptr;          // pinned staging of packed eigenvectors
  size_t zstage_cap = 0;
  long long launches = 0;
  Ctx() {
    hss_default_config(&cfg);
    memset(&stats, 0, sizeof stats);
  }
};

static Ctx &ctx() {
  static Ctx *c = new Ctx();
  return *c;
}

struct CudaError {
  std::string msg;
};

#define CK(x)                                                                       \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess) {                                                        \
      char b_[256];                                                                 \
      snprintf(b_, sizeof b_, "%s:%d %s: %s", __FILE__, __LINE__, #x,               \
               cudaGetErrorString(e_));                                             \
      throw CudaError{b_};                                                          \
    }                                                                               \
  } while (0)

template <class T>
static T *buf(Ctx &c, const char *name, size_t count) {
  Buf &b = c.bufs[name];
  size_t bytes = std::max<size_t>(count * sizeof(T), 256);
  if (b.cap < bytes) {
    if (b.p) {
      CK(cudaDeviceSynchronize());
      CK(cudaFree(b.p));
      b.p = nullptr;
      b.cap = 0;
    }
    size_t cap = bytes + bytes / 8;
    CK(cudaMalloc(&b.p, cap));
    b.cap = cap;
  }
  return (T *)b.p;
}

// sets the packed-output request for the duration of one solve
struct PzScope {
  Ctx &c;
  PzScope(Ctx &c_, PackedZ *p) : c(c_) { c.pz = p; }
  ~PzScope() { c.pz = nullptr; }
};

// pinned staging for packed eigenvectors (grows, kept)
static double *zstage(Ctx &c, size_t count) {
  if (c.zstage_cap < count) {
    if (c.zstage) CK(cudaFreeHost(c.zstage));
    c.zstage = nullptr;
    c.zstage_cap = 0;
    const size_t cap = count + count / 8;
    CK(cudaMallocHost((void **)&c.zstage, cap * sizeof(double)));
    c.zstage_cap = cap;
  }
  return c.zstage;
}

static void *pinned(Ctx &c, size_t bytes) {
  if (c.pinned_cap < bytes) {
    if (c.pinned) CK(cudaFreeHost(c.pinned));
    c.pinned = nullptr;
    size_t cap = std::max<size_t>(bytes * 2, 1 << 16);
    CK(cudaMallocHost(&c.pinned, cap));
    c.pinned_cap = cap;
  }
  return c.pinned;
}

void *pool_get(const char *name, size_t bytes) { return buf<char>(ctx(), name, bytes); }
// error word of the tensor-core products (set by a CTA whose bounded wait
// timed out; reset at the start of every solve, read with its status)
static int *gemm_flag(Ctx &c) { return buf<int>(c, "gemm_err", 1); }

// Host->device parameter uploads (level views, product descriptors).  Small
// ones stay pageable copies (measured faster: they travel with the command
// stream); the larger lists of the batched levels go through a pinned ring --
// a host memcpy plus an asynchronous copy, instead of a pageable copy that the
// driver may serialise with the stream.  Each ring region is reused only
// after the event recorded behind the copy that read it, normally long done.
void stage_h2d(void *dst, const void *src, size_t bytes, void *stream) {
  if (bytes == 0) return;
  Ctx &c = ctx();
  cudaStream_t st = (cudaStream_t)stream;
  constexpr size_t RING = 64u << 20;
  if (bytes <= (64u << 10) || bytes > RING / 4) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return;
  }
  if (!c.ring) {
    CK(cudaMallocHost((void **)&c.ring, RING));
    c.ring_cap = RING;
    c.ring_head = 0;
  }
  const size_t need = (bytes + 255) & ~(size_t)255;
  if (c.ring_head + need > c.ring_cap) c.ring_head = 0;
  const size_t a = c.ring_head, b = a + need;
  // the oldest uses come first; wait for (and retire) those [a, b) overlaps
  while (!c.ring_uses.empty() && c.ring_uses.front().a < b && a < c.ring_uses.front().b) {
    CK(cudaEventSynchronize(c.ring_uses.front().ev));
    c.ring_ev.push_back(c.ring_uses.front().ev);
    c.ring_uses.pop_front();
  }
  char *p = c.ring + a;
  memcpy(p, src, bytes);
  CK(cudaMemcpyAsync(dst, p, bytes, cudaMemcpyHostToDevice, st));
  cudaEvent_t ev;
  if (c.ring_ev.empty()) {
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  } else {
    ev = c.ring_ev.back();
    c.ring_ev.pop_back();
  }
  CK(cudaEventRecord(ev, st));
  c.ring_uses.push_back({a, b, ev});
  c.ring_head = b;
}

static cudaEvent_t next_event(Ctx &c) {
  if (c.evused == c.evpool.size()) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c.evpool.push_back(e);
  }
  return c.evpool[c.evused++];
}

void stage_begin(int stage, void *st) {
  Ctx &c = ctx();
  if (!c.cfg.profile) return;
  cudaEvent_t a = next_event(c);
  CK(cudaEventRecord(a, (cudaStream_t)st));
  c.open_ev[stage] = a;
}

void stage_end(int stage, void *st, long long bytes, double flops) {
  Ctx &c = ctx();
  c.stats.stage_bytes[stage] += bytes;
  c.stats.stage_flops[stage] += flops;
  if (!c.cfg.profile || !c.open_ev[stage]) return;
  cudaEvent_t b = next_event(c);
  CK(cudaEventRecord(b, (cudaStream_t)st));
  c.ranges.push_back({stage, c.open_ev[stage], b, bytes, flops});
  c.open_ev[stage] = nullptr;
}

static void collect_stage_times(Ctx &c) {
  for (auto &r : c.ranges) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, r.a, r.b));
    c.stats.stage_ms[r.stage] += ms;
    c.stats.stage_calls[r.stage] += 1;
  }
  c.ranges.clear();
  c.evused = 0;
}

template <class T>
static void h2d(T *dst, const std::vector<T> &src, cudaStream_t st) {
  if (!src.empty()) stage_h2d(dst, src.data(), src.size() * sizeof(T), st);
}

// ------------------------------------------------------------- DC block --
struct MergeLevel {
  std::vector<int> s, n, n1;
};

// Level arrays shared by all stages of one level (length = block size n).
struct LevelArrays {
  int n = 0;
  LevelScratch w;
  double *lam, *difl, *difr, *zhat, *alpha;
  int *iters;
  int2 *sup = nullptr;  // per slot rows holding data (tridiagonal path; Q not zero-filled)
};

static LevelArrays level_arrays(Ctx &c, int n) {
  LevelArrays a;
  a.n = n;
  a.w.srt = buf<int>(c, "srt", n);
  a.w.ds = buf<double>(c, "ds", n);
  a.w.zs = buf<double>(c, "zs", n);
  a.w.typ = buf<unsigned char>(c, "typ", n);
  a.w.cand = buf<int>(c, "cand", n);
  a.w.dl = buf<double>(c, "dl", n);
  a.w.zw = buf<double>(c, "zw", n);
  a.w.ndslot = buf<int>(c, "ndslot", n);
  a.w.grp = buf<int>(c, "grp", n);
  a.w.dfslot = buf<int>(c, "dfslot", n);
  a.w.dfval = buf<double>(c, "dfval", n);
  a.w.gvp = buf<int>(c, "gvp", n);
  a.w.gvq = buf<int>(c, "gvq", n);
  a.w.gvc = buf<double>(c, "gvc", n);
  a.w.gvs = buf<double>(c, "gvs", n);
  a.w.l1slot = buf<int>(c, "l1slot", n);
  a.w.l2slot = buf<int>(c, "l2slot", n);
  a.w.l1val = buf<double>(c, "l1val", n);
  a.w.l2val = buf<double>(c, "l2val", n);
  a.lam = buf<double>(c, "lam", n);
  a.difl = buf<double>(c, "difl", n);
  a.difr = buf<double>(c, "difr", n);
  a.zhat = buf<double>(c, "zhat", n);
  a.alpha = buf<double>(c, "alpha", n);
  a.iters = buf<int>(c, "iters", n);
  return a;
}

// Host arrays of one phase packed into a single upload: each call of a
// pageable host->device copy costs microseconds of host time while the GPU
// waits at a level boundary; one copy per phase replaces a dozen.
struct Pack {
  std::vector<char> h;
  template <class T>
  size_t add(const std::vector<T> &v) {
    const size_t off = (h.size() + 15) & ~(size_t)15;
    h.resize(off + v.size() * sizeof(T));
    if (!v.empty()) memcpy(h.data() + off, v.data(), v.size() * sizeof(T));
    return off;
  }
  char *upload(Ctx &c, const char *name, cudaStream_t st) {
    char *d = buf<char>(c, name, std::max<size_t>(h.size(), 16));
    stage_h2d(d, h.data(), h.size(), st);
    return d;
  }
};

// One of the kd rank-one updates of a banded merge (the loop of MDSBED1,
// SRC/mdsbed1.f90): z per slot (a column of Z = Q^T W), the coupling rho_in
// per merge of the group, prepare flags, and the columns of Z still to come,
// which follow the update's Givens rotations and eigenvector matrix.
struct BandUpdate {
  const double *z = nullptr;
  const double *rho = nullptr;
  int flags = 0;
  double *zrest = nullptr;
  int nrest = 0;
  long long zld = 0;
};

// Process a group of merges of one level (all of them when batched, one when
// not).  Arrays ms/mn/mn1 describe the group.  bu: a banded rank-one update
// (null for the tridiagonal merge).
static void run_merges(Ctx &c, const std::vector<int> &ms, const std::vector<int> &mn,
                       const std::vector<int> &mn1, const double *e, double *Q, long long ldq,
                       double *Dp, int *perm, LevelArrays &L, int *status, cudaStream_t st,
                       const BandUpdate *bu = nullptr) {
  const int P = (int)ms.size();
  if (P == 0) return;
  // ---- upload the group and prepare (deflation)
  int pflags = bu ? bu->flags : 0;
  std::vector<int> poff(P + 1, 0);
  for (int m = 0; m < P; ++m) poff[m + 1] = poff[m] + mn[m];
  Pack pk0;
  const size_t o_ms = pk0.add(ms), o_mn = pk0.add(mn), o_mn1 = pk0.add(mn1), o_po = pk0.add(poff);
  char *d0 = pk0.upload(c, "g_pack", st);
  int *dms = (int *)(d0 + o_ms), *dmn = (int *)(d0 + o_mn), *dmn1 = (int *)(d0 + o_mn1);
  int *dout = buf<int>(c, "g_out", 5 * P);
  double *drho = buf<double>(c, "g_rho", P);
  stage_begin(HSS_ST_PREPARE, st);
  if (!(pflags & PREP_SORTED)) {
    // merged order and z for every position of the level in one wide launch
    int *dpo = (int *)(d0 + o_po);
    launch_merge_front(P, poff[P], dpo, dms, dmn, dmn1, e, Q, ldq, Dp, perm, L.w,
                       bu ? bu->z : nullptr, bu ? bu->rho : nullptr, pflags, st, L.sup);
    pflags |= PREP_FRONT;
    c.launches++;
  }
  launch_merge_prepare(P, *std::max_element(mn.begin(), mn.end()), dms, dmn, dmn1, e, Q, ldq, Dp,
                       perm, L.w, dout, drho, st, bu ? bu->z : nullptr, bu ? bu->rho : nullptr,
                       pflags, L.sup);
  {
    long long nn = 0;
    for (int x : mn) nn += x;
    // merged order + z row gather + compaction: ~64 bytes per position
    stage_end(HSS_ST_PREPARE, st, 64 * nn, 0.0);
  }
  c.launches++;
  char *hp = (char *)pinned(c, (size_t)P * (5 * sizeof(int) + sizeof(double)));
  int *hout = (int *)hp;
  double *hrho = (double *)(hp + (size_t)P * 5 * sizeof(int));
  CK(cudaMemcpyAsync(hout, dout, (size_t)P * 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hrho, drho, (size_t)P * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  // ---- plan
  std::vector<int> as, an, aK, aoff(1, 0), gs, gn, gng;
  std::vector<double> arho;
  std::vector<int> ds_, dn_, dK_, doff(1, 0);
  std::vector<double> drho_;
  std::vector<long long> q2off, soff, toff;
  std::vector<int> hsel;  // HSS merges (index into active arrays)
  for (auto *v : {&as, &an, &aK, &aoff, &gs, &gn, &gng, &ds_, &dn_, &dK_, &doff}) v->reserve(P + 1);
  for (auto *v : {&arho, &drho_}) v->reserve(P);
  for (auto *v : {&q2off, &soff}) v->reserve(P);
  long long q2tot = 0, stot = 0;
  int maxn = 0, maxn_g = 0;
  for (int m = 0; m < P; ++m) {
    const int K = hout[5 * m], ng = hout[5 * m + 1];
    c.stats.n_merges++;
    c.stats.total_k += K;
    c.stats.max_k = std::max(c.stats.max_k, K);
    if (ng > 0) { gs.push_back(ms[m]); gn.push_back(mn[m]); gng.push_back(ng); maxn_g = std::max(maxn_g, mn[m]); }
    if (K == 0) continue;
    as.push_back(ms[m]); an.push_back(mn[m]); aK.push_back(K); arho.push_back(hrho[m]);
    aoff.push_back(aoff.back() + K);
    maxn = std::max(maxn, mn[m]);
    const bool use_hss = K >= c.cfg.bsmlz;
    if (use_hss) {
      hsel.push_back((int)as.size() - 1);
      c.stats.n_hss_merges++;
      continue;
    }
    c.stats.n_dense_merges++;
    ds_.push_back(ms[m]); dn_.push_back(mn[m]); dK_.push_back(K); drho_.push_back(hrho[m]);
    doff.push_back(doff.back() + K);
    q2off.push_back(q2tot);
    q2tot += (long long)mn[m] * K;
    soff.push_back(stot);
    stot += (long long)K * K;
  }
  const int PA = (int)as.size();
  // every array the level's launches read, in one upload
  std::vector<int> apoff(PA + 1, 0);
  for (int a = 0; a < PA; ++a) apoff[a + 1] = apoff[a] + an[a];
  Pack pk;
  const size_t o_gs = pk.add(gs), o_gn = pk.add(gn), o_gng = pk.add(gng);
  const size_t o_as = pk.add(as), o_aK = pk.add(aK), o_aoff = pk.add(aoff), o_arho = pk.add(arho),
               o_apoff = pk.add(apoff);
  const size_t o_ds = pk.add(ds_), o_dK = pk.add(dK_), o_doff = pk.add(doff), o_drho = pk.add(drho_),
               o_dn = pk.add(dn_), o_q2 = pk.add(q2off), o_so = pk.add(soff);
  char *dpk = pk.upload(c, "l_pack", st);
  // ---- Givens rotations of deflation
  if (!gs.empty()) {
    int *g1 = (int *)(dpk + o_gs), *g2 = (int *)(dpk + o_gn), *g3 = (int *)(dpk + o_gng);
    stage_begin(HSS_ST_GIVENS, st);
    launch_widen((int)gs.size(), maxn_g, g1, g2, g3, L.w, Q, ldq, L.sup, st);
    launch_givens((int)gs.size(), maxn_g, g1, g2, g3, L.w, Q, ldq, st, bu ? bu->zrest : nullptr,
                  bu ? bu->nrest : 0, bu ? bu->zld : 0);
    long long gb = 0;
    for (size_t i = 0; i < gs.size(); ++i) gb += 32LL * gn[i] * gng[i];
    stage_end(HSS_ST_GIVENS, st, gb, 0.0);
    c.launches++;
  }
  if (PA == 0) return;
  // ---- secular equation + Loewner for every active merge
  int *vs = (int *)(dpk + o_as), *vK = (int *)(dpk + o_aK), *voff = (int *)(dpk + o_aoff);
  double *vrho = (double *)(dpk + o_arho);
  LevelView lv{vs, vK, vrho, voff, PA};
  const int total = aoff.back();
  c.stats.secular_roots += total;
  double k2 = 0.0;
  for (int K : aK) k2 += (double)K * K;
  float *guess = nullptr;
  const int maxK = *std::max_element(aK.begin(), aK.end());
  float4 *gref = nullptr;
  if (c.cfg.predictor >= 2) {
    // starts from an FP32 pre-solve of every root (3: refined by one
    // float-float step, exact starts in gref)
    guess = buf<float>(c, "guess", L.n);
    float *d32 = buf<float>(c, "pole_f32", L.n), *z32 = buf<float>(c, "z_f32", L.n);
    float *d32lo = nullptr, *z2h = nullptr, *z2l = nullptr;
    if (c.cfg.predictor == 3) {
      d32lo = buf<float>(c, "pole_f32lo", L.n);
      z2h = buf<float>(c, "z2_f32", L.n);
      z2l = buf<float>(c, "z2_f32lo", L.n);
      gref = buf<float4>(c, "guess_ref", L.n);
    }
    stage_begin(HSS_ST_PREDICT, st);
    launch_secular_guess32(lv, total, maxK, L.n, L.w.dl, L.w.zw, d32, z32, guess, st, false,
                           d32lo, z2h, z2l, gref);
    stage_end(HSS_ST_PREDICT, st, 0, 0.0);
    c.launches += 2;
  } else if (c.cfg.predictor && c.pred_ready) {
    // features for every position of the level (unused slots carry side = -1)
    float *feat = buf<float>(c, "pred_feat", (size_t)L.n * (mlp_nfeat() + 1));
    guess = buf<float>(c, "guess", L.n);
    stage_begin(HSS_ST_SECULAR, st);
    launch_secular_mid(lv, total, *std::max_element(aK.begin(), aK.end()), L.w.dl, L.w.zw, feat, st);
    stage_end(HSS_ST_SECULAR, st, 0, 0.0);
    stage_begin(HSS_ST_PREDICT, st);
    launch_predict(L.n, feat, buf<char>(c, "pred_wb", 0), buf<float>(c, "pred_norm", 0), guess, st);
    stage_end(HSS_ST_PREDICT, st, 0, 0.0);
    c.launches += 2;
  }
  stage_begin(HSS_ST_SECULAR, st);
  launch_secular(lv, total, maxK, L.w.dl, L.w.zw, L.lam, L.difl, L.difr, L.iters, status,
                 (unsigned long long *)(status + 2), guess, st, false, c.cfg.predictor >= 2, gref);
  // per pole term per evaluation: 2 sub, 1 div, 2 mul, 3 add (x ~4 evaluations)
  stage_end(HSS_ST_SECULAR, st, 40LL * total, 0.0);  // flops from the pole-term count
  stage_begin(HSS_ST_LOWNER, st);
  launch_lowner(lv, total, L.w.dl, L.difl, L.difr, L.w.zw, L.zhat, st, false,
                *std::max_element(aK.begin(), aK.end()));
  stage_end(HSS_ST_LOWNER, st, 40LL * total, 5.0 * k2);
  c.launches += 2;
  if (bu && bu->nrest > 0) {
    // the remaining Z columns follow the new eigenvectors (mdsbed4.f90:266-268)
    double *zt = buf<double>(c, "band_zt", (size_t)bu->nrest * bu->zld);
    stage_begin(HSS_ST_OTHER, st);
    launch_alpha(lv, total, L.w.dl, L.difl, L.difr, L.zhat, L.alpha, st);
    launch_band_zupdate(lv, total, L.w.dl, L.difl, L.difr, L.zhat, L.alpha, L.w.ndslot, bu->zrest,
                        bu->nrest, bu->zld, zt, st);
    stage_end(HSS_ST_OTHER, st, 0, (2.0 + 4.0 * bu->nrest) * k2);
    c.launches += 3;
  }
  // ---- dense merges: S, gather, GEMM (block structured), scatter
  const int PD = (int)ds_.size();
  if (PD > 0) {
    int *xs = (int *)(dpk + o_ds), *xK = (int *)(dpk + o_dK), *xoff = (int *)(dpk + o_doff),
        *xn = (int *)(dpk + o_dn);
    double *xrho = (double *)(dpk + o_drho);
    long long *xq2 = (long long *)(dpk + o_q2), *xso = (long long *)(dpk + o_so);
    LevelView dv{xs, xK, xrho, xoff, PD};
    const int dtot = doff.back();
    double *Q2 = buf<double>(c, "Q2", q2tot), *T = buf<double>(c, "T", q2tot);
    double *S = buf<double>(c, "S", stot);
    stage_begin(HSS_ST_BUILD_S, st);
    launch_build_S(dv, dtot, L.w.dl, L.difl, L.difr, L.zhat, L.w.grp, xso, S, st);
    stage_end(HSS_ST_BUILD_S, st, 8LL * stot * 2, 0.0);
    int maxnd = *std::max_element(dn_.begin(), dn_.end());
    stage_begin(HSS_ST_GATHER, st);
    launch_gather(PD, dtot, maxnd, xs, xn, xoff, L.w.ndslot, L.w.grp, xq2, Q, ldq, Q2, st, L.sup);
    stage_end(HSS_ST_GATHER, st, 16LL * q2tot, 0.0);
    // GEMM problems: top rows use type 1,2 columns, bottom rows type 2,3
    std::vector<GemmDesc> probs;
    probs.reserve(2 * (size_t)PD);
    int tiles = 0;
    int di = 0;
    for (int m = 0; m < P; ++m) {
      const int K = hout[5 * m];
      if (K == 0 || K >= c.cfg.bsmlz) continue;
      const int c1 = hout[5 * m + 2], c2 = hout[5 * m + 3];
      const int n = mn[m], n1 = mn1[m];
      double *q2 = Q2 + q2off[di], *t = T + q2off[di], *sm = S + soff[di];
      GemmDesc top{q2, sm, t, n, K, n, n1, K, c1 + c2, 0, tiles};
      tiles += gemm_tiles(n1, K);
      probs.push_back(top);
      GemmDesc bot{q2 + n1 + (long long)c1 * n, sm + c1, t + n1, n, K, n, n - n1, K, K - c1, 0, tiles};
      tiles += gemm_tiles(n - n1, K);
      probs.push_back(bot);
      ++di;
    }
    double fl = 0.0;
    long long gbytes = 0;
    for (auto &p : probs) {
      fl += 2.0 * p.M * p.N * p.K;
      gbytes += 8LL * ((long long)p.M * p.K + (long long)p.K * p.N + (long long)p.M * p.N);
    }
    stage_begin(HSS_ST_GEMM, st);
    launch_gemm(probs, c.cfg.precision, st);
    stage_end(HSS_ST_GEMM, st, gbytes, fl);
    stage_begin(HSS_ST_SCATTER, st);
    launch_scatter(PD, dtot, maxnd, xs, xn, xoff, L.w.ndslot, xq2, T, Q, ldq, st, L.sup);
    stage_end(HSS_ST_SCATTER, st, 16LL * q2tot, 0.0);
    c.launches += 4;
  }
  // ---- HSS merges: one at a time (each has its own HSS tree)
  for (int a : hsel) {
    HssMergeArgs h;
    h.s = as[a]; h.n = an[a]; h.K = aK[a];
    h.leaf = c.cfg.hss_leaf; h.tol = c.cfg.tol; h.precision = c.cfg.precision;
    h.dl = L.w.dl + h.s; h.difl = L.difl + h.s; h.difr = L.difr + h.s; h.zhat = L.zhat + h.s;
    h.alpha = L.alpha + h.s; h.ndslot = L.w.ndslot + h.s;
    h.Q = Q; h.ldq = ldq; h.sup = L.sup;
    int rank = 0;
    c.launches += hss_merge(h, &rank, st);  // times its own stages
    c.stats.max_rank = std::max(c.stats.max_rank, rank);
  }
  // ---- new ascending order and eigenvalues of the rewritten slots
  stage_begin(HSS_ST_FINISH, st);
  launch_merge_finish_grid(PA, apoff[PA], (int *)(dpk + o_apoff), vs, vK, L.lam, L.w, perm, Dp, st);
  {
    long long nn = 0;
    for (int x : an) nn += x;
    stage_end(HSS_ST_FINISH, st, 24 * nn, 0.0);
  }
  c.launches++;
}

// Eigen-decomposition of many unreduced, scaled blocks at once.  Block b
// covers global positions bs[b] .. bs[b] + bm[b] - 1 of d, e, Dp, perm and the
// same rows and columns of Q (leading dim ldq); e is zero at every block's last
// position, so no cut crosses two blocks.  Each block is halved down to leaves
// of at most smlsiz; the leaves of all blocks form one launch and the merges of
// one tree level of all blocks are processed together.
static void dc_blocks(Ctx &c, const std::vector<int> &bs, const std::vector<int> &bm, int N,
                      const double *d, const double *e, double *Q, long long ldq, double *Dp,
                      int *perm, int *status, cudaStream_t st, int2 *sup) {
  const int smlsiz = std::max(1, std::min(c.cfg.smlsiz, 32));
  const int nb = (int)bs.size();
  std::vector<std::vector<int>> ends(nb);
  std::vector<int> ls, lz;
  int mmax = 1;
  double fl = 0.0;
  for (int b = 0; b < nb; ++b) {
    std::vector<int> sz(1, bm[b]);
    while (*std::max_element(sz.begin(), sz.end()) > smlsiz) {
      std::vector<int> nx;
      for (int x : sz) { nx.push_back(x / 2); nx.push_back((x + 1) / 2); }
      sz.swap(nx);
    }
    int acc = bs[b];
    for (int x : sz) {
      ls.push_back(acc); lz.push_back(x);
      acc += x;
      ends[b].push_back(acc);
      mmax = std::max(mmax, x);
      fl += 30.0 * x * x * x;
    }
  }
  const int nl = (int)ls.size();
  int *dls = buf<int>(c, "leaf_s", nl), *dlz = buf<int>(c, "leaf_z", nl);
  h2d(dls, ls, st); h2d(dlz, lz, st);
  stage_begin(HSS_ST_LEAF, st);
  launch_leaf(nl, dls, dlz, mmax, N, d, e, Q, ldq, Dp, perm, status, st, sup);
  stage_end(HSS_ST_LEAF, st, 8LL * N * smlsiz, fl);
  c.launches++;
  bool more = false;
  for (auto &v : ends) more |= v.size() > 1;
  if (!more) return;
  LevelArrays L = level_arrays(c, N);
  L.sup = sup;
  while (more) {
    MergeLevel lvl;
    more = false;
    for (int b = 0; b < nb; ++b) {
      std::vector<int> &en = ends[b];
      if (en.size() < 2) continue;
      std::vector<int> nx;
      for (size_t i = 0; i + 1 < en.size(); i += 2) {
        const int s = i == 0 ? bs[b] : en[i - 1];
        lvl.s.push_back(s); lvl.n.push_back(en[i + 1] - s); lvl.n1.push_back(en[i] - s);
        nx.push_back(en[i + 1]);
      }
      en.swap(nx);
      more |= en.size() > 1;
    }
    c.stats.n_levels++;
    if (c.cfg.batched) {
      run_merges(c, lvl.s, lvl.n, lvl.n1, e, Q, ldq, Dp, perm, L, status, st);
    } else {
      for (size_t m = 0; m < lvl.s.size(); ++m)
        run_merges(c, {lvl.s[m]}, {lvl.n[m]}, {lvl.n1[m]}, e, Q, ldq, Dp, perm, L, status, st);
    }
  }
}

// One tridiagonal of a solve: host copies of d (n) and e (n - 1), device
// outputs z (leading dim ldz) and w (n eigenvalues, ascending).
struct Problem {
  int n;
  const double *hd, *he;
  double *z;
  long long ldz;
  double *w;
};

// MDSTEDC('I') of every problem in one pass over the DC tree levels.  Problem
// p occupies global positions P[p] .. P[p+1] - 1; all problems share one Q of
// leading dimension L = max n_p, problem p's block starting at Q + P[p](L + 1).
// Within a problem: split on tiny E and scale each unreduced block
// (mdstedc.f90:305-345), DC on every block, then order the eigenpairs
// (mdstedc.f90:392-420).
static int solve_core(Ctx &c, const std::vector<Problem> &pr, cudaStream_t st) {
  memset(&c.stats, 0, sizeof c.stats);
  c.launches = 0;
  cudaEvent_t ev0, ev1;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  CK(cudaEventRecord(ev0, st));
  const int np = (int)pr.size();
  std::vector<long long> P(np + 1, 0);
  long long L = 1;
  for (int p = 0; p < np; ++p) {
    P[p + 1] = P[p] + pr[p].n;
    L = std::max<long long>(L, pr[p].n);
  }
  const int N = (int)P[np];
  if (N == 0) return 0;
  const size_t qsize = (size_t)(N - 1) * (size_t)(L + 1) + 1;
  double *Q = buf<double>(c, "Q", qsize);
  double *Dp = buf<double>(c, "Dp", N);
  int *perm = buf<int>(c, "perm", N);
  double *d = buf<double>(c, "d_in", N), *e = buf<double>(c, "e_in", N);
  long long *dP = nullptr;
  // status[0]: error code, status[2..3]: 64-bit sum of secular iterations,
  // status[4..5]: 64-bit count of learned starts that fell back, status[6..7]:
  // 64-bit sum over roots of iterations x K (pole terms evaluated)
  int *status = buf<int>(c, "status", 8);
  CK(cudaMemsetAsync(status, 0, 8 * sizeof(int), st));
  CK(cudaMemsetAsync(gemm_flag(c), 0, sizeof(int), st));
  // no zero fill of Q: every column is tracked with the rows it holds data on
  // (set by the leaves, widened by merges) and read as zero elsewhere
  int2 *sup = buf<int2>(c, "sup", N);
  if (np > 1) {
    dP = buf<long long>(c, "prob_P", np + 1);
    h2d(dP, P, st);
  }
  // global d, e with e = 0 at every block end; split and scale per problem
  std::vector<double> hd(N), he(N, 0.0);
  std::vector<int> bstart, bsize, bprob;
  std::vector<double> bscale;
  std::vector<int> nblocks(np, 0);
  const int smlsiz = std::max(1, std::min(c.cfg.smlsiz, 32));
  struct Blocks {
    std::vector<int> start, size, prob;
    std::vector<double> scale;
  };
  // problems p0 .. p1 - 1 into their own block lists (problems touch disjoint
  // ranges of hd, he and nblocks, so ranges of problems run on separate threads)
  auto split = [&](int p0, int p1, Blocks &out) {
    for (int p = p0; p < p1; ++p) {
      const int n = pr[p].n, o = (int)P[p];
      for (int i = 0; i < n; ++i) hd[o + i] = pr[p].hd[i];
      for (int i = 0; i + 1 < n; ++i) he[o + i] = pr[p].he[i];
      int start = o;
      while (start < o + n) {
        int finish = start;
        while (finish < o + n - 1 && !negligible(he[finish], hd[finish], hd[finish + 1])) ++finish;
        he[finish] = 0.0;
        double nrm = 0.0;
        for (int i = start; i <= finish; ++i) nrm = std::max(nrm, std::fabs(hd[i]));
        for (int i = start; i < finish; ++i) nrm = std::max(nrm, std::fabs(he[i]));
        const int m = finish - start + 1;
        double scl = 1.0;
        if (m > smlsiz && nrm > 0.0) {
          scl = nrm;
          const double mul = 1.0 / nrm;
          for (int i = start; i <= finish; ++i) hd[i] *= mul;
          for (int i = start; i < finish; ++i) he[i] *= mul;
        }
        out.start.push_back(start); out.size.push_back(m); out.scale.push_back(scl);
        out.prob.push_back(p);
        nblocks[p]++;
        start = finish + 1;
      }
    }
  };
  {
    // a batch of many positions splits on host threads, each taking a run of
    // whole problems of about N / nt positions; the lists join in problem order
    const int nt = N >= (1 << 17) && np > 1 ? std::min(host_threads(), np) : 1;
    std::vector<Blocks> part(nt);
    std::vector<int> cut(nt + 1, np);
    cut[0] = 0;
    for (int t = 1, p = 0; t < nt; ++t) {
      const long long goal = (long long)N * t / nt;
      while (p < np && P[p] < goal) ++p;
      cut[t] = std::max(p, cut[t - 1]);
    }
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) {
      try {
        th.emplace_back(split, cut[t], cut[t + 1], std::ref(part[t]));
      } catch (...) {
        split(cut[t], cut[t + 1], part[t]);  // no thread available: run it here
      }
    }
    split(cut[0], cut[1], part[0]);
    for (auto &x : th) x.join();
    for (const Blocks &b : part) {
      bstart.insert(bstart.end(), b.start.begin(), b.start.end());
      bsize.insert(bsize.end(), b.size.begin(), b.size.end());
      bscale.insert(bscale.end(), b.scale.begin(), b.scale.end());
      bprob.insert(bprob.end(), b.prob.begin(), b.prob.end());
    }
  }
  CK(cudaMemcpyAsync(d, hd.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(e, he.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
  dc_blocks(c, bstart, bsize, N, d, e, Q, L, Dp, perm, status, st, sup);
  {
    std::vector<int> ss, sm;
    std::vector<double> sc;
    for (size_t b = 0; b < bstart.size(); ++b)
      if (bscale[b] != 1.0) { ss.push_back(bstart[b]); sm.push_back(bsize[b]); sc.push_back(bscale[b]); }
    if (!ss.empty()) {
      int *x1 = buf<int>(c, "scl_s", ss.size()), *x2 = buf<int>(c, "scl_m", ss.size());
      double *x3 = buf<double>(c, "scl_v", sc.size());
      h2d(x1, ss, st); h2d(x2, sm, st); h2d(x3, sc, st);
      launch_scale_blocks((int)ss.size(), x1, x2, x3, Dp, st);
      c.launches++;
    }
  }
  // problems split into several blocks: merge the blocks' ascending lists
  int *fperm = perm;
  if (*std::max_element(nblocks.begin(), nblocks.end()) > 1) {
    std::vector<int> hp(N);
    std::vector<double> hv(N);
    CK(cudaMemcpyAsync(hp.data(), perm, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hv.data(), Dp, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int p = 0; p < np; ++p) {
      if (nblocks[p] < 2) continue;
      std::vector<std::pair<double, int>> all;
      all.reserve(pr[p].n);
      // perm holds global slots; Dp is indexed by slot
      for (long long i = P[p]; i < P[p + 1]; ++i) all.push_back({hv[hp[i]], hp[i]});
      std::stable_sort(all.begin(), all.end(),
                       [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
                         return a.first < b.first;
                       });
      for (size_t i = 0; i < all.size(); ++i) hp[P[p] + i] = all[i].second;
    }
    fperm = buf<int>(c, "fperm", N);
    h2d(fperm, hp, st);
  }
  stage_begin(HSS_ST_FINAL, st);
  long long final_bytes = 0;
  bool packed = false;
  if (np == 1 && c.pz && c.pz->want && sup) {
    // output column i is slot fperm[i], holding data on rows sup[slot]
    PackedZ &pz = *c.pz;
    std::vector<int> hp(N);
    std::vector<int2> hs(N);
    CK(cudaMemcpyAsync(hp.data(), fperm, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hs.data(), sup, sizeof(int2) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    pz.seg.resize(N);
    pz.off.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) {
      const int2 r = hs[hp[i]];
      pz.seg[i] = r;
      pz.off[i + 1] = pz.off[i] + std::max(0, r.y - r.x);
    }
    pz.total = pz.off[N];
    // supports cover at most 60 % of Z, and the pinned staging stays <= 4 GB
    if (pz.total * 5 <= (long long)N * N * 3 && pz.total <= (4LL << 30) / 8) {
      long long *doff = buf<long long>(c, "pz_off", N + 1);
      stage_h2d(doff, pz.off.data(), sizeof(long long) * (N + 1), st);
      pz.dbuf = buf<double>(c, "pz_data", (size_t)std::max<long long>(pz.total, 1));
      launch_pack_columns(N, fperm, Dp, Q, L, sup, doff, pz.dbuf, pr[0].w, st);
      pz.packed = packed = true;
      final_bytes = 16LL * pz.total + 20LL * N;
    }
  }
  if (packed) {
    // the packed segments replace the n x n write
  } else if (np == 1) {
    launch_final_gather(N, fperm, Dp, Q, L, pr[0].z, pr[0].ldz, pr[0].w, st, sup);
  } else {
    std::vector<double *> hz(np), hw(np);
    std::vector<long long> hl(np);
    for (int p = 0; p < np; ++p) { hz[p] = pr[p].z; hw[p] = pr[p].w; hl[p] = pr[p].ldz; }
    double **dz = buf<double *>(c, "prob_z", np), **dw = buf<double *>(c, "prob_w", np);
    long long *dl = buf<long long>(c, "prob_ldz", np);
    h2d(dz, hz, st); h2d(dw, hw, st); h2d(dl, hl, st);
    launch_final_gather_batch(np, N, dP, fperm, Dp, Q, L, dz, dl, dw, st, sup);
  }
  {
    long long nn = 0;
    for (auto &q : pr) nn += (long long)q.n * q.n;
    // compulsory traffic: the n^2 output write and the slot/eigenvalue
    // vectors; the Q reads cover only the columns' supports (data dependent)
    stage_end(HSS_ST_FINAL, st, packed ? final_bytes : 8LL * nn + 20LL * N, 0.0);
  }
  c.launches++;
  CK(cudaEventRecord(ev1, st));
  int hst[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(hst, status, sizeof hst, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hst + 1, gemm_flag(c), sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const int hstatus = hst[0];
  unsigned long long its, fb;
  memcpy(&its, hst + 2, sizeof its);
  memcpy(&fb, hst + 4, sizeof fb);
  c.stats.secular_iters = (long long)its;
  c.stats.predictor_fallbacks = (long long)fb;
  {
    // per pole term per evaluation: 2 subtractions, a reciprocal (estimate +
    // 3 fma = 6 flops), a multiply and 2 fma
    unsigned long long terms;
    memcpy(&terms, hst + 6, sizeof terms);
    c.stats.stage_flops[HSS_ST_SECULAR] = 13.0 * (double)terms;
  }
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ev0, ev1));
  c.stats.ms_total = ms;
  c.stats.kernel_launches = c.launches;
  collect_stage_times(c);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  CK(cudaGetLastError());
  if (hst[1]) {
    c.err = "tensor-core product: bounded wait timed out";
    return 1;
  }
  if (hstatus != 0) {
    c.err = hstatus == HSS_SECULAR_NOCONV ? "secular iteration did not converge"
                                           : "leaf QL iteration did not converge";
    return 1;
  }
  return 0;
}

static int mdstedc_core(Ctx &c, int n, const std::vector<double> &hd, const std::vector<double> &he,
                        double *dz, long long ldz, double *dw, cudaStream_t st);

// ------------------------------------------------------------ band DC ----
// MDSBEVD('I', 'U') (SRC/mdsbevd.f90:183) of one symmetric band matrix in HBM:
// ab in upper band storage (ldab >= kd + 1), 2 <= kd <= 32.  Halving tree to
// leaves of at most max(smlsiz, 2 kd) rows; every cut split by the SVD of its
// coupling block; dense leaf eigensolves; then per level kd rank-one updates
// of all merges of the level (MDSBED1, SRC/mdsbed1.f90:2).  z (ldz) and w
// (ascending) are the outputs.
static int band_core(Ctx &c, int n, int kd, const double *ab, long long ldab, double *z,
                     long long ldz, double *w, cudaStream_t st) {
  memset(&c.stats, 0, sizeof c.stats);
  c.launches = 0;
  cudaEvent_t ev0, ev1;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  CK(cudaEventRecord(ev0, st));
  const int bound = std::min(64, std::max(std::max(1, std::min(c.cfg.smlsiz, 64)), 2 * kd));
  std::vector<int> sz(1, n);
  while (*std::max_element(sz.begin(), sz.end()) > bound) {
    std::vector<int> nx;
    for (int x : sz) { nx.push_back(x / 2); nx.push_back((x + 1) / 2); }
    sz.swap(nx);
  }
  const int nl = (int)sz.size(), ncut = nl - 1;
  std::vector<int> ls(nl), ends(nl), cabove(nl), cbelow(nl), crow(std::max(ncut, 1));
  int mmax = 1;
  for (int i = 0, acc = 0; i < nl; ++i) {
    ls[i] = acc;
    acc += sz[i];
    ends[i] = acc;
    mmax = std::max(mmax, sz[i]);
    cabove[i] = i > 0 ? i - 1 : -1;
    cbelow[i] = i < nl - 1 ? i : -1;
    if (i < nl - 1) crow[i] = acc - 1;
  }
  double *Q = buf<double>(c, "Q", (size_t)n * n);
  double *Dp = buf<double>(c, "Dp", n);
  int *perm = buf<int>(c, "perm", n);
  int *status = buf<int>(c, "status", 8);
  CK(cudaMemsetAsync(status, 0, 8 * sizeof(int), st));
  CK(cudaMemsetAsync(gemm_flag(c), 0, sizeof(int), st));
  CK(cudaMemsetAsync(Q, 0, sizeof(double) * (size_t)n * n, st));
  const size_t kk = (size_t)kd * kd;
  double *Uc = buf<double>(c, "band_U", std::max<size_t>(ncut, 1) * kk);
  double *Vc = buf<double>(c, "band_V", std::max<size_t>(ncut, 1) * kk);
  double *Sc = buf<double>(c, "band_S", std::max<size_t>(ncut, 1) * kd);
  int *dcrow = buf<int>(c, "band_crow", crow.size());
  int *dls = buf<int>(c, "leaf_s", nl), *dlz = buf<int>(c, "leaf_z", nl);
  int *dca = buf<int>(c, "band_ca", nl), *dcb = buf<int>(c, "band_cb", nl);
  h2d(dcrow, crow, st); h2d(dls, ls, st); h2d(dlz, sz, st); h2d(dca, cabove, st);
  h2d(dcb, cbelow, st);
  stage_begin(HSS_ST_LEAF, st);
  launch_band_cut_svd(ncut, dcrow, kd, ab, ldab, Uc, Vc, Sc, status, st);
  launch_band_leaf(nl, dls, dlz, dca, dcb, mmax, kd, ab, ldab, Uc, Vc, Sc, Q, n, Dp, perm, status,
                   st);
  {
    double fl = 0.0;
    for (int x : sz) fl += 8.0 * x * x * x * 10.0;  // ~10 Jacobi sweeps
    stage_end(HSS_ST_LEAF, st, 8LL * n * (kd + 1), fl);
  }
  c.launches += 2;
  if (nl > 1) {
    std::vector<double> hS((size_t)ncut * kd);
    CK(cudaMemcpyAsync(hS.data(), Sc, sizeof(double) * hS.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    LevelArrays L = level_arrays(c, n);
    double *Z = buf<double>(c, "band_Z", (size_t)kd * n);
    std::vector<int> lastleaf(nl);
    for (int i = 0; i < nl; ++i) lastleaf[i] = i;
    while (ends.size() > 1) {
      std::vector<int> ms, mn, mn1, mcut, nxe, nxl;
      for (size_t i = 0; i + 1 < ends.size(); i += 2) {
        const int s = i == 0 ? 0 : ends[i - 1];
        ms.push_back(s); mn.push_back(ends[i + 1] - s); mn1.push_back(ends[i] - s);
        mcut.push_back(lastleaf[i]);
        nxe.push_back(ends[i + 1]);
        nxl.push_back(lastleaf[i + 1]);
      }
      const int P = (int)ms.size();
      c.stats.n_levels++;
      int *zs = buf<int>(c, "bz_s", P), *zn = buf<int>(c, "bz_n", P), *zn1 = buf<int>(c, "bz_n1", P),
          *zc = buf<int>(c, "bz_c", P);
      h2d(zs, ms, st); h2d(zn, mn, st); h2d(zn1, mn1, st); h2d(zc, mcut, st);
      stage_begin(HSS_ST_PREPARE, st);
      launch_band_z(P, *std::max_element(mn.begin(), mn.end()), zs, zn, zn1, zc, kd, Q, n, Uc, Vc, Z,
                    n, st);
      stage_end(HSS_ST_PREPARE, st, 8LL * n * kd * 2, 2.0 * n * kd * kd);
      c.launches++;
      double *drho = buf<double>(c, "band_rho", (size_t)P * kd);
      std::vector<double> hr((size_t)P * kd);
      for (int k = 0; k < kd; ++k)
        for (int m = 0; m < P; ++m) hr[(size_t)k * P + m] = hS[(size_t)mcut[m] * kd + k];
      h2d(drho, hr, st);
      for (int k = 0; k < kd; ++k) {
        BandUpdate bu;
        bu.flags = k == 0 ? 0 : (PREP_SORTED | PREP_DENSE);
        bu.z = Z + (size_t)k * n;
        bu.zrest = Z + (size_t)(k + 1) * n;
        bu.nrest = kd - k - 1;
        bu.zld = n;
        if (c.cfg.batched) {
          bu.rho = drho + (size_t)k * P;
          run_merges(c, ms, mn, mn1, nullptr, Q, n, Dp, perm, L, status, st, &bu);
        } else {
          for (int m = 0; m < P; ++m) {
            bu.rho = drho + (size_t)k * P + m;
            run_merges(c, {ms[m]}, {mn[m]}, {mn1[m]}, nullptr, Q, n, Dp, perm, L, status, st, &bu);
          }
        }
      }
      ends.swap(nxe);
      lastleaf.swap(nxl);
    }
  }
  stage_begin(HSS_ST_FINAL, st);
  launch_final_gather(n, perm, Dp, Q, n, z, ldz, w, st);
  stage_end(HSS_ST_FINAL, st, 16LL * n * n + 20LL * n, 0.0);
  c.launches++;
  CK(cudaEventRecord(ev1, st));
  int hst[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(hst, status, sizeof hst, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hst + 1, gemm_flag(c), sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  unsigned long long its, fb;
  memcpy(&its, hst + 2, sizeof its);
  memcpy(&fb, hst + 4, sizeof fb);
  c.stats.secular_iters = (long long)its;
  c.stats.predictor_fallbacks = (long long)fb;
  {
    // per pole term per evaluation: 2 subtractions, a reciprocal (estimate +
    // 3 fma = 6 flops), a multiply and 2 fma
    unsigned long long terms;
    memcpy(&terms, hst + 6, sizeof terms);
    c.stats.stage_flops[HSS_ST_SECULAR] = 13.0 * (double)terms;
  }
  float ms_ = 0.f;
  CK(cudaEventElapsedTime(&ms_, ev0, ev1));
  c.stats.ms_total = ms_;
  c.stats.kernel_launches = c.launches;
  collect_stage_times(c);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  CK(cudaGetLastError());
  if (hst[1]) {
    c.err = "tensor-core product: bounded wait timed out";
    return 1;
  }
  if (hst[0] != 0) {
    c.err = hst[0] == HSS_SECULAR_NOCONV ? "secular iteration did not converge"
                                          : "leaf Jacobi iteration did not converge";
    return 1;
  }
  return 0;
}

__global__ void k_scale(int n, double *x, double a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] *= a;
}

// ------------------------------------------------------------- SVD DC ----
// The part of a level of SVD merges after their deflation (shared by the
// bidiagonal merges and the banded row appends): the deflating rotations of U
// and V columns, the secular equation and the z rebuild in squared mode, the
// K x K U and V blocks, the products U2 Ub and V2 Vb (DLASD3's products) or the
// HSS products (DHSSVCS), sigma back to scale and the new ascending order.
// hout: the prepare's 5 ints per merge (pinned); mpos: positions per merge
// (the arrow's size, the pole first); mN / mM: rows of U / V in its window
// [ms, ms + mN) / [ms, ms + mM); dms / dpos: ms and mpos on the device.
static void svd_merge_tail(Ctx &c, const std::vector<int> &ms, const std::vector<int> &mpos,
                           const std::vector<int> &mN, const std::vector<int> &mM,
                           const int *dms, const int *dpos, const int *hout, const double *dnrm,
                           double *U, double *V, long long ld, double *Dp, int *perm,
                           LevelArrays &L, int *status, cudaStream_t st) {
  const int P = (int)ms.size();
  const int maxPos = *std::max_element(mpos.begin(), mpos.end());
  std::vector<int> aK(P), aoff(P + 1, 0), gs, gN, gM, gng;
  std::vector<double> ones(P, 1.0);
  int maxK = 1, maxNg = 0, maxMg = 0;
  for (int m = 0; m < P; ++m) {
    const int K = hout[5 * m], ng = hout[5 * m + 1];
    aK[m] = K;
    aoff[m + 1] = aoff[m] + K;
    maxK = std::max(maxK, K);
    c.stats.n_merges++;
    c.stats.n_dense_merges++;
    c.stats.total_k += K;
    c.stats.max_k = std::max(c.stats.max_k, K);
    if (ng > 0) {
      gs.push_back(ms[m]); gN.push_back(mN[m]); gM.push_back(mM[m]); gng.push_back(ng);
      maxNg = std::max(maxNg, mN[m]); maxMg = std::max(maxMg, mM[m]);
    }
  }
  if (!gs.empty()) {  // deflating rotations of U columns and V columns (mdlasd2.f90)
    const int G = (int)gs.size();
    int *g1 = buf<int>(c, "sg_s", G), *g2 = buf<int>(c, "sg_N", G), *g3 = buf<int>(c, "sg_M", G),
        *g4 = buf<int>(c, "sg_g", G);
    h2d(g1, gs, st); h2d(g2, gN, st); h2d(g3, gM, st); h2d(g4, gng, st);
    stage_begin(HSS_ST_GIVENS, st);
    launch_givens(G, maxNg, g1, g2, g4, L.w, U, ld, st);
    launch_givens(G, maxMg, g1, g3, g4, L.w, V, ld, st);
    stage_end(HSS_ST_GIVENS, st, 0, 0.0);
    c.launches += 2;
  }
  int *vK = buf<int>(c, "sv_K", P), *voff = buf<int>(c, "sv_off", P + 1);
  double *vr = buf<double>(c, "sv_rho", P);
  h2d(vK, aK, st); h2d(voff, aoff, st); h2d(vr, ones, st);
  LevelView lv{dms, vK, vr, voff, P};
  const int total = aoff.back();
  c.stats.secular_roots += total;
  double k2 = 0.0;
  for (int K : aK) k2 += (double)K * K;
  float *guess = nullptr;
  float4 *gref = nullptr;
  if (c.cfg.predictor >= 2) {  // starts from an FP32 pre-solve in squared mode
    guess = buf<float>(c, "guess", L.n);
    float *d32 = buf<float>(c, "pole_f32", L.n), *z32 = buf<float>(c, "z_f32", L.n);
    float *d32lo = nullptr, *z2h = nullptr, *z2l = nullptr;
    if (c.cfg.predictor == 3) {
      d32lo = buf<float>(c, "pole_f32lo", L.n);
      z2h = buf<float>(c, "z2_f32", L.n);
      z2l = buf<float>(c, "z2_f32lo", L.n);
      gref = buf<float4>(c, "guess_ref", L.n);
    }
    stage_begin(HSS_ST_PREDICT, st);
    launch_secular_guess32(lv, total, maxK, L.n, L.w.dl, L.w.zw, d32, z32, guess, st, true,
                           d32lo, z2h, z2l, gref);
    stage_end(HSS_ST_PREDICT, st, 0, 0.0);
    c.launches += 2;
  }
  stage_begin(HSS_ST_SECULAR, st);
  launch_secular(lv, total, maxK, L.w.dl, L.w.zw, L.lam, L.difl, L.difr, L.iters, status,
                 (unsigned long long *)(status + 2), guess, st, true, guess != nullptr, gref);
  stage_end(HSS_ST_SECULAR, st, 40LL * total, 0.0);  // flops from the pole-term count
  stage_begin(HSS_ST_LOWNER, st);
  launch_lowner(lv, total, L.w.dl, L.difl, L.difr, L.w.zw, L.zhat, st, true, maxK);
  stage_end(HSS_ST_LOWNER, st, 40LL * total, 8.0 * k2);
  c.launches += 2;
  // ---- dense merges (K < bsmlz): K x K U / V blocks, batched GEMMs
  std::vector<int> ds_, dN_, dM_, dK_, doff_(1, 0);
  std::vector<long long> qU, qV, bo;
  long long totU = 0, totV = 0, totB = 0;
  int maxNd = 1, maxMd = 1;
  std::vector<int> hsel;
  for (int m = 0; m < P; ++m) {
    const int K = aK[m];
    if (K >= c.cfg.bsmlz) { hsel.push_back(m); continue; }
    ds_.push_back(ms[m]); dN_.push_back(mN[m]); dM_.push_back(mM[m]); dK_.push_back(K);
    doff_.push_back(doff_.back() + K);
    qU.push_back(totU); totU += (long long)mN[m] * K;
    qV.push_back(totV); totV += (long long)mM[m] * K;
    bo.push_back(totB); totB += (long long)K * K;
    maxNd = std::max(maxNd, mN[m]); maxMd = std::max(maxMd, mM[m]);
  }
  const int PD = (int)ds_.size();
  if (PD > 0) {
    int *xs = buf<int>(c, "svd_s", PD), *xN = buf<int>(c, "svd_N", PD), *xM = buf<int>(c, "svd_M", PD),
        *xK = buf<int>(c, "svd_K", PD), *xoff = buf<int>(c, "svd_off", PD + 1);
    long long *dqU = buf<long long>(c, "sv_qU", PD), *dqV = buf<long long>(c, "sv_qV", PD),
              *dbo = buf<long long>(c, "sv_bo", PD);
    h2d(xs, ds_, st); h2d(xN, dN_, st); h2d(xM, dM_, st); h2d(xK, dK_, st); h2d(xoff, doff_, st);
    h2d(dqU, qU, st); h2d(dqV, qV, st); h2d(dbo, bo, st);
    LevelView dv{xs, xK, vr, xoff, PD};
    const int dtot = doff_.back();
    double *Ub = buf<double>(c, "sv_Ub", totB), *Vb = buf<double>(c, "sv_Vb", totB);
    stage_begin(HSS_ST_BUILD_S, st);
    launch_svd_vectors(dv, dtot, L.w.dl, L.difl, L.difr, L.zhat, dbo, Ub, Vb, st);
    stage_end(HSS_ST_BUILD_S, st, 16LL * totB, 20.0 * k2);
    double *U2 = buf<double>(c, "sv_U2", totU), *TU = buf<double>(c, "sv_TU", totU);
    double *V2 = buf<double>(c, "sv_V2", totV), *TV = buf<double>(c, "sv_TV", totV);
    stage_begin(HSS_ST_GATHER, st);
    launch_gather(PD, dtot, maxNd, xs, xN, xoff, L.w.ndslot, nullptr, dqU, U, ld, U2, st);
    launch_gather(PD, dtot, maxMd, xs, xM, xoff, L.w.ndslot, nullptr, dqV, V, ld, V2, st);
    stage_end(HSS_ST_GATHER, st, 16LL * (totU + totV), 0.0);
    std::vector<GemmDesc> probs;
    int tiles = 0;
    double fl = 0.0;
    long long gb = 0;
    for (int m = 0; m < PD; ++m) {
      const int K = dK_[m], N = dN_[m], M = dM_[m];
      probs.push_back(GemmDesc{U2 + qU[m], Ub + bo[m], TU + qU[m], N, K, N, N, K, K, 0, tiles});
      tiles += gemm_tiles(N, K);
      probs.push_back(GemmDesc{V2 + qV[m], Vb + bo[m], TV + qV[m], M, K, M, M, K, K, 0, tiles});
      tiles += gemm_tiles(M, K);
      fl += 2.0 * (double)(N + M) * K * K;
      gb += 8LL * ((long long)(N + M) * K * 2 + 2LL * K * K);
    }
    stage_begin(HSS_ST_GEMM, st);
    launch_gemm(probs, c.cfg.precision, st);
    stage_end(HSS_ST_GEMM, st, gb, fl);
    stage_begin(HSS_ST_SCATTER, st);
    launch_scatter(PD, dtot, maxNd, xs, xN, xoff, L.w.ndslot, dqU, TU, U, ld, st);
    launch_scatter(PD, dtot, maxMd, xs, xM, xoff, L.w.ndslot, dqV, TV, V, ld, st);
    stage_end(HSS_ST_SCATTER, st, 16LL * (totU + totV), 0.0);
    c.launches += 6;
  }
  // ---- HSS merges (K >= bsmlz): two HSS products each (DHSSVCS)
  for (int m : hsel) {
    SvdHssArgs h;
    h.s = ms[m]; h.N = mN[m]; h.M = mM[m]; h.K = aK[m];
    h.leaf = c.cfg.hss_leaf; h.tol = c.cfg.tol; h.precision = c.cfg.precision;
    h.dl = L.w.dl + h.s; h.difl = L.difl + h.s; h.difr = L.difr + h.s; h.zhat = L.zhat + h.s;
    h.ndslot = L.w.ndslot + h.s;
    h.U = U; h.V = V; h.ld = ld;
    int rank = 0;
    c.launches += svd_hss_merge(h, &rank, st);
    c.stats.n_hss_merges++;
    c.stats.n_dense_merges--;
    c.stats.max_rank = std::max(c.stats.max_rank, rank);
  }
  // ---- sigma back to scale, new ascending order
  stage_begin(HSS_ST_FINISH, st);
  launch_svd_unscale(lv, total, dnrm, L.lam, st);
  launch_merge_finish(P, maxPos, dms, dpos, vK, L.lam, L.w, perm, Dp, st);
  stage_end(HSS_ST_FINISH, st, 0, 0.0);
  c.launches += 2;
}

// One level of bidiagonal SVD merges (MDLASD1, SRC/mdlasd1.f90): deflation
// (MDLASD2) by k_svd_prepare, then svd_merge_tail.  Merge m covers rows
// ms[m] .. ms[m] + N - 1, N = nl + 1 + nr.
static void run_svd_merges(Ctx &c, const std::vector<int> &ms, const std::vector<int> &mnl,
                           const std::vector<int> &mnr, const std::vector<int> &msq,
                           const double *d, const double *e, double *U, double *V, long long ld,
                           double *Dp, int *perm, LevelArrays &L, int *status, cudaStream_t st) {
  const int P = (int)ms.size();
  if (P == 0) return;
  std::vector<int> mN(P), mM(P);
  for (int m = 0; m < P; ++m) { mN[m] = mnl[m] + 1 + mnr[m]; mM[m] = mN[m] + msq[m]; }
  const int maxN = *std::max_element(mN.begin(), mN.end());
  int *dms = buf<int>(c, "sv_s", P), *dnl = buf<int>(c, "sv_nl", P), *dnr = buf<int>(c, "sv_nr", P),
      *dsq = buf<int>(c, "sv_sq", P), *dN = buf<int>(c, "sv_N", P);
  h2d(dms, ms, st); h2d(dnl, mnl, st); h2d(dnr, mnr, st); h2d(dsq, msq, st); h2d(dN, mN, st);
  int *dout = buf<int>(c, "g_out", 5 * P);
  double *dnrm = buf<double>(c, "sv_nrm", P);
  stage_begin(HSS_ST_PREPARE, st);
  launch_svd_prepare(P, maxN, dms, dnl, dnr, dsq, d, e, U, ld, V, ld, Dp, perm, L.w, dout, dnrm,
                     st);
  {
    long long nn = 0;
    for (int x : mN) nn += x;
    stage_end(HSS_ST_PREPARE, st, 64 * nn, 0.0);
  }
  c.launches++;
  int *hout = (int *)pinned(c, (size_t)P * 5 * sizeof(int));
  CK(cudaMemcpyAsync(hout, dout, (size_t)P * 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  svd_merge_tail(c, ms, mN, mN, mM, dms, dN, hout, dnrm, U, V, ld, Dp, perm, L, status, st);
}

// MDBDSDC('U', COMPQ) (SRC/mdbdsdc.f90:1) of the upper bidiagonal (d, e) in
// HBM: singular values into w (descending), U (ldu) and VT (ldvt) when
// vectors.  Tree as DLASDT: a node of N rows splits into nl = N/2 rows, the
// center row, and nr = N - nl - 1 rows, down to leaves of at most smlsiz
// rows; left children carry the center's column (sqre = 1).
static int svd_core(Ctx &c, int n, const double *d, const double *e, double *Uo, long long ldu,
                    double *VT, long long ldvt, double *w, bool vectors, cudaStream_t st) {
  memset(&c.stats, 0, sizeof c.stats);
  c.launches = 0;
  cudaEvent_t ev0, ev1;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  CK(cudaEventRecord(ev0, st));
  const int smlsiz = std::max(4, std::min(c.cfg.smlsiz, 32));
  // levels of nodes, root first: (start, rows, sqre)
  struct Node { int a, N, sq; };
  std::vector<std::vector<Node>> lv(1, std::vector<Node>{Node{0, n, 0}});
  while (true) {
    int mx = 0;
    for (auto &x : lv.back()) mx = std::max(mx, x.N);
    if (mx <= smlsiz) break;
    std::vector<Node> nx;
    for (auto &x : lv.back()) {
      const int nl = x.N / 2, nr = x.N - nl - 1;
      nx.push_back(Node{x.a, nl, 1});
      nx.push_back(Node{x.a + nl + 1, nr, x.sq});
    }
    lv.push_back(nx);
  }
  double *U = buf<double>(c, "sv_U", (size_t)n * n);
  double *V = buf<double>(c, "sv_V", (size_t)n * n);
  double *Dp = buf<double>(c, "Dp", n);
  int *perm = buf<int>(c, "perm", n);
  int *status = buf<int>(c, "status", 8);
  CK(cudaMemsetAsync(status, 0, 8 * sizeof(int), st));
  CK(cudaMemsetAsync(gemm_flag(c), 0, sizeof(int), st));
  CK(cudaMemsetAsync(U, 0, sizeof(double) * (size_t)n * n, st));
  CK(cudaMemsetAsync(V, 0, sizeof(double) * (size_t)n * n, st));
  {
    const std::vector<Node> &leaves = lv.back();
    std::vector<int> ls, lz, lq;
    int rmax = 1;
    double flops = 0.0;
    for (auto &x : leaves) {
      ls.push_back(x.a); lz.push_back(x.N); lq.push_back(x.sq);
      rmax = std::max(rmax, x.N);
      flops += 40.0 * x.N * x.N * x.N;
    }
    const int nl = (int)ls.size();
    int *dls = buf<int>(c, "leaf_s", nl), *dlz = buf<int>(c, "leaf_z", nl), *dlq = buf<int>(c, "leaf_q", nl);
    h2d(dls, ls, st); h2d(dlz, lz, st); h2d(dlq, lq, st);
    stage_begin(HSS_ST_LEAF, st);
    launch_svd_leaf(nl, dls, dlz, dlq, rmax, d, e, U, n, V, n, Dp, perm, status, st);
    stage_end(HSS_ST_LEAF, st, 16LL * n * smlsiz, flops);
    c.launches++;
  }
  if (lv.size() > 1) {
    LevelArrays L = level_arrays(c, n);
    for (int k = (int)lv.size() - 2; k >= 0; --k) {  // merges bottom-up
      std::vector<int> ms, mnl, mnr, msq;
      for (auto &x : lv[k]) {
        const int nl = x.N / 2;
        ms.push_back(x.a); mnl.push_back(nl); mnr.push_back(x.N - nl - 1); msq.push_back(x.sq);
      }
      c.stats.n_levels++;
      if (c.cfg.batched) {
        run_svd_merges(c, ms, mnl, mnr, msq, d, e, U, V, n, Dp, perm, L, status, st);
      } else {
        for (size_t m = 0; m < ms.size(); ++m)
          run_svd_merges(c, {ms[m]}, {mnl[m]}, {mnr[m]}, {msq[m]}, d, e, U, V, n, Dp, perm, L,
                         status, st);
      }
    }
  }
  stage_begin(HSS_ST_FINAL, st);
  launch_svd_outputs(n, perm, Dp, U, n, V, n, Uo, ldu, VT, ldvt, w, vectors, st);
  stage_end(HSS_ST_FINAL, st, vectors ? 32LL * n * n : 16LL * n, 0.0);
  c.launches += 2;
  CK(cudaEventRecord(ev1, st));
  int hst[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(hst, status, sizeof hst, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hst + 1, gemm_flag(c), sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  unsigned long long its, terms;
  memcpy(&its, hst + 2, sizeof its);
  memcpy(&terms, hst + 6, sizeof terms);
  c.stats.secular_iters = (long long)its;
  // squared poles: one more multiply and add per term
  c.stats.stage_flops[HSS_ST_SECULAR] = 15.0 * (double)terms;
  float ms_ = 0.f;
  CK(cudaEventElapsedTime(&ms_, ev0, ev1));
  c.stats.ms_total = ms_;
  c.stats.kernel_launches = c.launches;
  collect_stage_times(c);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  CK(cudaGetLastError());
  if (hst[1]) {
    c.err = "tensor-core product: bounded wait timed out";
    return 1;
  }
  if (hst[0] != 0) {
    c.err = hst[0] == HSS_SECULAR_NOCONV ? "secular iteration did not converge"
                                          : "leaf SVD iteration did not converge";
    return 1;
  }
  return 0;
}

// Host front end of MDBDSDC (SRC/mdbdsdc.f90): lower bidiagonal rotated to upper
// (the DLARTG loop), scaling by max |d|, |e|, the device solve, the rotations
// applied back to U (DLASR), the scale undone.  hd/he: host copies.
static int svd_solve(Ctx &c, bool lower, int n, std::vector<double> hd, std::vector<double> he,
                     double *dU, long long ldu, double *dVT, long long ldvt, double *dw,
                     bool vectors, cudaStream_t st) {
  he.resize(std::max(n, 1), 0.0);
  std::vector<double> cs, sn;
  if (lower) {
    cs.resize(std::max(n - 1, 1)); sn.resize(std::max(n - 1, 1));
    for (int i = 0; i + 1 < n; ++i) {
      const double f = hd[i], g = he[i];
      const double r = std::hypot(f, g);
      const double cc = r == 0.0 ? 1.0 : f / r, ss = r == 0.0 ? 0.0 : g / r;
      hd[i] = r;
      he[i] = ss * hd[i + 1];
      hd[i + 1] = cc * hd[i + 1];
      cs[i] = cc;
      sn[i] = -ss;
    }
  }
  double nrm = 0.0;
  for (int i = 0; i < n; ++i) nrm = std::max(nrm, std::fabs(hd[i]));
  for (int i = 0; i + 1 < n; ++i) nrm = std::max(nrm, std::fabs(he[i]));
  const double scl = nrm > 0.0 ? nrm : 1.0;
  for (int i = 0; i < n; ++i) hd[i] /= scl;
  for (int i = 0; i + 1 < n; ++i) he[i] /= scl;
  double *d = buf<double>(c, "svd_d", n), *e = buf<double>(c, "svd_e", std::max(n, 1));
  CK(cudaMemcpyAsync(d, hd.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(e, he.data(), sizeof(double) * he.size(), cudaMemcpyHostToDevice, st));
  const int info = svd_core(c, n, d, e, dU, ldu, dVT, ldvt, dw, vectors, st);
  k_scale<<<(n + 255) / 256, 256, 0, st>>>(n, dw, scl);
  if (lower && vectors) {
    double *dcs = buf<double>(c, "svd_cs", cs.size()), *dsn = buf<double>(c, "svd_sn", sn.size());
    h2d(dcs, cs, st); h2d(dsn, sn, st);
    launch_rows_rotate_back(n, n, dcs, dsn, dU, ldu, st);
  }
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  return info;
}

// ------------------------------------------------------ banded SVD DC ----
// MDBDSVDT (SRC/mdbdsvdt.f90): a node of X rows keeps nl = X / 2 rows on the
// left, sb center rows and nr = X - nl - sb rows on the right; the left child
// has sb extra columns, the right child those of its parent (the root none).
// lv[0 .. depth - 1] are the merge levels (root first), lv[depth] the leaves.
struct BNode {
  int s, X, sq;  // rows [s, s + X), sq extra columns (0 or sb)
  int nl;        // rows of the left child (merge nodes)
};

// balanced: nl = (X - sb + 1) / 2 instead of X / 2 (both sides within one row)
static bool bsvd_levels(int n, int sb, int depth, bool balanced,
                        std::vector<std::vector<BNode>> &lv) {
  lv.assign(1, std::vector<BNode>{BNode{0, n, 0, 0}});
  for (int d = 0; d < depth; ++d) {
    std::vector<BNode> nx;
    for (BNode &x : lv.back()) {
      const int nl = balanced ? (x.X - sb + 1) / 2 : x.X / 2, nr = x.X - nl - sb;
      if (nl < 1 || nr < 1) return false;
      x.nl = nl;
      nx.push_back(BNode{x.s, nl, sb, 0});
      nx.push_back(BNode{x.s + nl + sb, nr, x.sq, 0});
    }
    lv.push_back(nx);
  }
  return true;
}

// The reference's depth floor(log2(n / (msub + 1))) (at least 1), made valid
// (every node keeps rows on both sides), then deepened until every leaf has at
// most 32 rows (the leaf Jacobi's cost grows as c^2 (r + c) and its warps work
// along the rows), or, where no tree gets there (sb near 32), 64 rows (one
// CTA's shared memory, bsvd_rows_max()).  The reference's halving shrinks
// right children by sb at every level; when no depth of it fits, balanced cuts
// are used instead.  Returns the depth, or -1.
static int bsvd_tree(int n, int sb, int msub, std::vector<std::vector<BNode>> &lv) {
  auto largest = [&lv]() {
    int mx = 0;
    for (const BNode &x : lv.back()) mx = std::max(mx, x.X);
    return mx;
  };
  for (const int cap : {std::min(32, bsvd_rows_max()), bsvd_rows_max()}) {
    if (n <= cap) {
      lv.assign(1, std::vector<BNode>{BNode{0, n, 0, 0}});
      return 0;
    }
    for (int balanced = 0; balanced < 2; ++balanced) {
      int depth = balanced ? 1 : std::max(1, (int)std::floor(std::log2((double)n / (double)(msub + 1))));
      while (depth > 1 && !bsvd_levels(n, sb, depth, balanced, lv)) --depth;
      if (!bsvd_levels(n, sb, depth, balanced, lv)) continue;
      bool fits = true;
      while (fits && largest() > cap) {
        std::vector<std::vector<BNode>> t;
        fits = bsvd_levels(n, sb, depth + 1, balanced, t);
        if (fits) {
          lv.swap(t);
          ++depth;
        }
      }
      if (fits) return depth;
    }
  }
  return -1;
}

// Append k (0 .. sb - 1) of every merge of one level (MDBDSVD1's loop over the
// inserted rows, SRC/mdbdsvd1.f90:259-354): z = V^T b for row c_k = s + nl + k,
// the fold of the null vectors, the deflation, then the shared merge tail.
static void run_bsvd_append(Ctx &c, const std::vector<BNode> &nodes, int k, int sb, int n,
                            const double *ab, long long ldab, double *U, double *V, long long ld,
                            double *Dp, int *perm, LevelArrays &L, int *status, cudaStream_t st) {
  const int P = (int)nodes.size();
  std::vector<int> ms(P), mrow(P), mN(P), mM(P), mnl(P), mna(P), mb0(P), mnb(P), mpos(P),
      poff(P + 1, 0);
  for (int m = 0; m < P; ++m) {
    const BNode &x = nodes[m];
    const int nl = x.nl, nr = x.X - nl - sb;
    ms[m] = x.s;
    mN[m] = x.X;
    mM[m] = x.X + x.sq;
    mnl[m] = nl;
    mrow[m] = x.s + nl + k;
    mna[m] = k == 0 ? nl : nl + nr + k;  // the first append merges both children's lists
    mb0[m] = k == 0 ? x.s + nl + sb : 0;
    mnb[m] = k == 0 ? nr : 0;
    mpos[m] = nl + nr + k + 1;
    poff[m + 1] = poff[m] + mM[m];
  }
  const int maxM = *std::max_element(mM.begin(), mM.end());
  const int maxPos = *std::max_element(mpos.begin(), mpos.end());
  int *dms = buf<int>(c, "bs_s", P), *drow = buf<int>(c, "bs_row", P), *dN = buf<int>(c, "bs_N", P),
      *dM = buf<int>(c, "bs_M", P), *dnl = buf<int>(c, "bs_nl", P), *dna = buf<int>(c, "bs_na", P),
      *db0 = buf<int>(c, "bs_b0", P), *dnb = buf<int>(c, "bs_nb", P), *dpos = buf<int>(c, "bs_pos", P),
      *dpoff = buf<int>(c, "bs_poff", P + 1);
  h2d(dms, ms, st); h2d(drow, mrow, st); h2d(dN, mN, st); h2d(dM, mM, st); h2d(dnl, mnl, st);
  h2d(dna, mna, st); h2d(db0, mb0, st); h2d(dnb, mnb, st); h2d(dpos, mpos, st); h2d(dpoff, poff, st);
  double *z = buf<double>(c, "bs_z", n);
  double *amax = buf<double>(c, "bs_amax", P);
  int *dout = buf<int>(c, "g_out", 5 * P);
  double *dnrm = buf<double>(c, "sv_nrm", P);
  stage_begin(HSS_ST_PREPARE, st);
  launch_bsvd_z(P, poff[P], dpoff, dms, drow, sb, n, ab, ldab, V, ld, z, st);
  launch_bsvd_fold(P, maxM, dms, dN, dM, dnl, drow, sb, n, ab, ldab, V, ld, z, amax, st);
  launch_bsvd_prepare(P, maxPos, dms, drow, dna, db0, dnb, amax, z, U, ld, Dp, perm, L.w, dout,
                      dnrm, st);
  {
    long long bytes = 0;
    for (int m = 0; m < P; ++m)
      bytes += 8LL * mM[m] * (sb + 2) + 16LL * mM[m] * (2 * sb) + 64LL * mpos[m];
    stage_end(HSS_ST_PREPARE, st, bytes, 0.0);
  }
  c.launches += 3;
  int *hout = (int *)pinned(c, (size_t)P * 5 * sizeof(int));
  CK(cudaMemcpyAsync(hout, dout, (size_t)P * 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  svd_merge_tail(c, ms, mpos, mN, mM, dms, dpos, hout, dnrm, U, V, ld, Dp, perm, L, status, st);
}

// MDBDSVD (SRC/mdbdsvd.f90:1) of the n x n upper banded matrix in HBM (upper
// band storage, ldab >= sb + 1): singular values descending into w, U (ldu),
// VT (ldvt).  The leaves' dense SVDs, then per merge level the sb row appends.
static int bsvd_core(Ctx &c, int n, int sb, const double *ab, long long ldab, int msub,
                     double *Uo, long long ldu, double *VT, long long ldvt, double *w,
                     cudaStream_t st) {
  memset(&c.stats, 0, sizeof c.stats);
  c.launches = 0;
  std::vector<std::vector<BNode>> lv;
  const int depth = bsvd_tree(n, sb, msub, lv);
  if (depth < 0) {
    c.err = "MDBDSVD: no cut of the band leaves every block within the leaf size";
    return -2;
  }
  cudaEvent_t ev0, ev1;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  CK(cudaEventRecord(ev0, st));
  double *U = buf<double>(c, "sv_U", (size_t)n * n);
  double *V = buf<double>(c, "sv_V", (size_t)n * n);
  double *Dp = buf<double>(c, "Dp", n);
  int *perm = buf<int>(c, "perm", n);
  int *status = buf<int>(c, "status", 8);
  CK(cudaMemsetAsync(status, 0, 8 * sizeof(int), st));
  CK(cudaMemsetAsync(gemm_flag(c), 0, sizeof(int), st));
  CK(cudaMemsetAsync(U, 0, sizeof(double) * (size_t)n * n, st));
  CK(cudaMemsetAsync(V, 0, sizeof(double) * (size_t)n * n, st));
  {
    std::vector<int> la, lr, lc;
    double flops = 0.0;
    for (const BNode &x : lv.back()) {
      la.push_back(x.s);
      lr.push_back(x.X);
      lc.push_back(x.X + x.sq);
      const double cc = x.X + x.sq;
      flops += 10.0 * 3.0 * cc * cc * (x.X + cc);  // ~10 sweeps of c^2/2 rotations
    }
    const int nl = (int)la.size();
    int *dla = buf<int>(c, "bl_a", nl), *dlr = buf<int>(c, "bl_r", nl), *dlc = buf<int>(c, "bl_c", nl);
    h2d(dla, la, st); h2d(dlr, lr, st); h2d(dlc, lc, st);
    stage_begin(HSS_ST_LEAF, st);
    launch_bsvd_leaf(nl, dla, dlr, dlc, sb, ab, ldab, U, n, V, n, Dp, perm, status, st);
    stage_end(HSS_ST_LEAF, st, 8LL * n * (sb + 1) + 16LL * n * 96, flops);
    c.launches++;
  }
  if (depth > 0) {
    LevelArrays L = level_arrays(c, n);
    for (int d = depth - 1; d >= 0; --d) {  // merges bottom-up
      c.stats.n_levels++;
      for (int k = 0; k < sb; ++k)
        run_bsvd_append(c, lv[d], k, sb, n, ab, ldab, U, V, n, Dp, perm, L, status, st);
    }
  }
  stage_begin(HSS_ST_FINAL, st);
  launch_svd_outputs(n, perm, Dp, U, n, V, n, Uo, ldu, VT, ldvt, w, true, st);
  stage_end(HSS_ST_FINAL, st, 32LL * n * n, 0.0);
  c.launches += 2;
  CK(cudaEventRecord(ev1, st));
  int hst[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(hst, status, sizeof hst, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hst + 1, gemm_flag(c), sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  unsigned long long its, terms;
  memcpy(&its, hst + 2, sizeof its);
  memcpy(&terms, hst + 6, sizeof terms);
  c.stats.secular_iters = (long long)its;
  c.stats.stage_flops[HSS_ST_SECULAR] = 15.0 * (double)terms;
  float ms_ = 0.f;
  CK(cudaEventElapsedTime(&ms_, ev0, ev1));
  c.stats.ms_total = ms_;
  c.stats.kernel_launches = c.launches;
  collect_stage_times(c);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  CK(cudaGetLastError());
  if (hst[1]) {
    c.err = "tensor-core product: bounded wait timed out";
    return 1;
  }
  if (hst[0] != 0) {
    c.err = hst[0] == HSS_SECULAR_NOCONV ? "secular iteration did not converge"
                                          : "leaf Jacobi iteration did not converge";
    return 1;
  }
  return 0;
}

// Symmetric band eigensolve from device arrays: ab upper band storage
// (ldab >= kd + 1).  kd <= 1 is a tridiagonal and goes through the
// tridiagonal solver; 2 <= kd <= 32 through band_core.
// Band -> tridiagonal on the device (band_sbr.cu), then the tridiagonal
// divide and conquer; with eigenvectors, Z = Q Z_T by applying the reduction's
// reflectors to the tridiagonal's eigenvectors.  The reference takes this
// route (LAPACK DSBTRD + DSTERF / DSBEVD) for eigenvalues only and for KD > 16
// (SRC/mdsbedc.f90:274-276, :311-318); here it serves eigenvalues only and the
// bandwidths above the band divide and conquer's limit.  ab: upper storage.
static int band_sbr_solve(Ctx &c, int n, int kd, const double *ab, long long ldab, double *z,
                          long long ldz, double *w, bool wantz, cudaStream_t st) {
  const int b = std::min(kd, n - 1);
  if (b > 4096) {
    c.err = "band reduction: bandwidth above 4096";
    return -4;
  }
  const int ldb = 2 * b;
  double *LB = buf<double>(c, "sbr_band", (size_t)ldb * n);
  launch_sbr_load(n, kd, b, ab, ldab, LB, ldb, st);
  std::vector<long long> roff;
  const long long nref = sbr_reflectors(n, b, &roff);
  double *R = nullptr, *rtau = nullptr;
  long long *droff = nullptr;
  if (wantz && nref > 0) {
    R = buf<double>(c, "sbr_v", (size_t)nref * b);
    rtau = buf<double>(c, "sbr_tau", (size_t)nref);
    droff = buf<long long>(c, "sbr_roff", roff.size());
    stage_h2d(droff, roff.data(), sizeof(long long) * roff.size(), st);
  }
  const int nl = launch_sbr_reduce(n, b, LB, ldb, R, droff, rtau, st);
  double *dd = buf<double>(c, "sbr_d", n), *de = buf<double>(c, "sbr_e", n);
  launch_sbr_tri(n, LB, ldb, dd, de, st);
  std::vector<double> hd(n), he(n, 0.0);
  CK(cudaMemcpyAsync(hd.data(), dd, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(he.data(), de, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  double *zt = wantz ? z : buf<double>(c, "z_scratch", (size_t)n * n);
  const int info = mdstedc_core(c, n, hd, he, zt, wantz ? ldz : n, w, st);
  if (info != 0) return info;
  int nb = 0;
  if (wantz && nref > 0) nb = launch_sbr_back(n, b, R, droff, rtau, z, ldz, st);
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  c.launches += nl + nb + 2;
  c.stats.kernel_launches = c.launches;
  return 0;
}

static int band_solve(Ctx &c, int n, int kd, const double *ab, long long ldab, double *z,
                      long long ldz, double *w, cudaStream_t st, bool wantz = true) {
  if (kd >= 2 && n > 2 && (kd > HSS_BAND_KD_MAX || !wantz))
    return band_sbr_solve(c, n, kd, ab, ldab, z, ldz, w, wantz, st);
  if (kd <= 1 || n <= 2) {
    std::vector<double> hab((size_t)ldab * n);
    CK(cudaMemcpyAsync(hab.data(), ab, sizeof(double) * hab.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<double> hd(n), he(std::max(n, 1), 0.0);
    for (int j = 0; j < n; ++j) hd[j] = hab[(size_t)j * ldab + kd];
    if (kd >= 1)
      for (int j = 1; j < n; ++j) he[j - 1] = hab[(size_t)j * ldab + kd - 1];
    return mdstedc_core(c, n, hd, he, z, ldz, w, st);
  }
  return band_core(c, n, kd, ab, ldab, z, ldz, w, st);
}

// MDSTEDC('I') of one matrix.  hd/he: host copies of d/e (n, n-1).
static int mdstedc_core(Ctx &c, int n, const std::vector<double> &hd, const std::vector<double> &he,
                        double *dz, long long ldz, double *dw, cudaStream_t st) {
  return solve_core(c, {Problem{n, hd.data(), he.data(), dz, ldz, dw}}, st);
}

// MDSTEDC('V') of one matrix: on entry z (n x n, ldz, device) holds the
// orthogonal matrix Q0 that reduced the original matrix to the tridiagonal
// (d, e) (DSYTRD + DORGTR, say); on exit Q0 * Q_T, Q_T the tridiagonal's
// eigenvectors in ascending eigenvalue order.  The reference multiplies Q0 into
// each split block's eigenvector matrix (SRC/mdstedc.f90:341-372: MDLAED0 with
// ICOMPQ = 1, or DSTEQR + DGEMM on small blocks) before its final ordering.
// Here the tridiagonal is solved once as for 'I', and Q0 is applied through
// the supports of the DC eigenvectors: output column c of Q_T holds data only
// on rows [x_c, y_c) (the range of the last merge that rewrote it), so columns
// sharing a range form one product Q0(:, x:y) * Q_T(x:y, cols); the products
// go to a scratch matrix in group order and are scattered back into z.  When
// the supports fill most of Q_T, one dense product Q0 * Q_T is used instead.
static int mdstedc_v_core(Ctx &c, int n, const std::vector<double> &hd,
                          const std::vector<double> &he, double *z, long long ldz, double *dw,
                          cudaStream_t st) {
  double *T = buf<double>(c, "v_prod", (size_t)n * n);
  PackedZ pz;
  pz.want = true;
  int info;
  {
    PzScope scope(c, &pz);
    // packed output when the supports are sparse; else Q_T itself lands in T
    info = mdstedc_core(c, n, hd, he, T, n, dw, st);
  }
  if (info != 0) return info;
  int *err = gemm_flag(c);
  CK(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (!pz.packed) {
    double *P = buf<double>(c, "v_dense", (size_t)n * n);
    std::vector<GemmDesc> p{{z, T, P, (int)ldz, n, n, n, n, n, 0, 0}};
    launch_gemm(p, c.cfg.precision, st);
    c.launches++;
    CK(cudaMemcpy2DAsync(z, sizeof(double) * ldz, P, sizeof(double) * n, sizeof(double) * n, n,
                         cudaMemcpyDeviceToDevice, st));
  } else {
    // output columns grouped by support segment (stable: output order within a group)
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      const int2 &ra = pz.seg[a], &rb = pz.seg[b];
      return ra.x != rb.x ? ra.x < rb.x : ra.y < rb.y;
    });
    std::vector<long long> doff(n + 1, 0);
    for (int j = 0; j < n; ++j) {
      const int2 r = pz.seg[order[j]];
      doff[j + 1] = doff[j] + std::max(0, r.y - r.x);
    }
    int *dorder = buf<int>(c, "v_order", n);
    long long *dsoff = buf<long long>(c, "v_soff", n + 1);
    long long *ddoff = buf<long long>(c, "v_doff", n + 1);
    double *B2 = buf<double>(c, "v_packed", (size_t)std::max<long long>(pz.total, 1));
    stage_h2d(dorder, order.data(), sizeof(int) * n, st);
    stage_h2d(dsoff, pz.off.data(), sizeof(long long) * (n + 1), st);
    stage_h2d(ddoff, doff.data(), sizeof(long long) * (n + 1), st);
    launch_repack_columns(n, dorder, dsoff, ddoff, pz.dbuf, B2, st);
    c.launches++;
    std::vector<GemmDesc> prods;
    for (int j0 = 0; j0 < n;) {
      const int2 r = pz.seg[order[j0]];
      int j1 = j0 + 1;
      while (j1 < n && pz.seg[order[j1]].x == r.x && pz.seg[order[j1]].y == r.y) ++j1;
      const int m = r.y - r.x;
      if (m > 0)
        prods.push_back(GemmDesc{z + (long long)r.x * ldz, B2 + doff[j0], T + (long long)j0 * n,
                                 (int)ldz, m, n, n, j1 - j0, m, 0, 0});
      else  // a column without support rows (cannot occur for an eigenvector)
        CK(cudaMemsetAsync(T + (long long)j0 * n, 0, sizeof(double) * n * (j1 - j0), st));
      j0 = j1;
    }
    launch_gemm(prods, c.cfg.precision, st);
    c.launches++;
    // z is free once the products have read it
    launch_scatter_columns(n, n, dorder, T, n, z, ldz, st);
    c.launches++;
  }
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  if (herr) {
    c.err = "tensor-core product: bounded wait timed out";
    return 1;
  }
  return 0;
}

// Message for hss_last_error() from entry points that live outside this file.
void set_last_error(const std::string &msg) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  c.err = msg;
}

}  // namespace hss

// ================================================================== C ABI ==
using namespace hss;

extern "C" {

void hss_default_config(hss_config *cfg) {
  memset(cfg, 0, sizeof *cfg);
  cfg->hss_leaf = 200;
  cfg->bsmlz = 1500;
  cfg->tol = 1e-17;
  cfg->smlsiz = 25;
  cfg->precision = 0;
  cfg->predictor = 0;
  cfg->batched = 1;
}

void hss_set_config(const hss_config *cfg) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  c.cfg = *cfg;
  set_secular_terms(cfg->sec_terms);
  set_split_min_log2(cfg->split_min_log2);
  set_small_nk(cfg->small_nk);
  set_split_min_m(cfg->split_min_m);
  set_secular_threads(cfg->sec_threads);
  set_gemm_path(cfg->gemm_path);
}
void hss_get_config(hss_config *cfg) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  *cfg = c.cfg;
}
void hss_get_stats(hss_stats *st) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  *st = c.stats;
}
const char *hss_last_error(void) { return ctx().err.c_str(); }

int hss_finalize(void) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  cudaDeviceSynchronize();
  for (auto &kv : c.bufs)
    if (kv.second.p) cudaFree(kv.second.p);
  c.bufs.clear();
  if (c.pinned) cudaFreeHost(c.pinned);
  c.pinned = nullptr;
  c.pinned_cap = 0;
  if (c.ring) cudaFreeHost(c.ring);
  c.ring = nullptr;
  c.ring_cap = c.ring_head = 0;
  for (auto &u : c.ring_uses) cudaEventDestroy(u.ev);
  c.ring_uses.clear();
  for (auto ev : c.ring_ev) cudaEventDestroy(ev);
  c.ring_ev.clear();
  if (c.zstage) cudaFreeHost(c.zstage);
  c.zstage = nullptr;
  c.zstage_cap = 0;
  return 0;
}

int hss_mdstedc_dev(int n, double *d, double *e, double *z, int ldz, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -2;
  if (ldz < std::max(1, n)) return -6;
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    std::vector<double> hd(n), he(std::max(n, 1), 0.0);
    CK(cudaMemcpyAsync(hd.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (n > 1) CK(cudaMemcpyAsync(he.data(), e, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double *dw = buf<double>(c, "w_out", n);
    int info = mdstedc_core(c, n, hd, he, z, ldz, dw, st);
    CK(cudaMemcpyAsync(d, dw, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    return info;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_mdstedc_v_dev(int n, double *d, double *e, double *z, int ldz, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -2;
  if (ldz < std::max(1, n)) return -6;
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    if (n == 1) {  // SRC/mdstedc.f90:248-251: Z(1,1) = 1
      const double one = 1.0;
      CK(cudaMemcpyAsync(z, &one, sizeof(double), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
      return 0;
    }
    std::vector<double> hd(n), he(n, 0.0);
    CK(cudaMemcpyAsync(hd.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(he.data(), e, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double *dw = buf<double>(c, "w_out", n);
    int info = mdstedc_v_core(c, n, hd, he, z, ldz, dw, st);
    CK(cudaMemcpyAsync(d, dw, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    return info;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_mdstedc_batch_dev(int nprob, const int *n, double *d, double *e, double *z, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (nprob < 0) return -1;
  if (nprob == 0) return 0;
  if (!n) return -2;
  long long N = 0, zz = 0;
  for (int p = 0; p < nprob; ++p) {
    if (n[p] < 0) {
      c.err = "hss_mdstedc_batch_dev: n[" + std::to_string(p) + "] < 0";
      return -2;
    }
    N += n[p];
    zz += (long long)n[p] * n[p];
  }
  if (N > 2147483647LL) {
    c.err = "hss_mdstedc_batch_dev: total order exceeds 2^31 - 1";
    return -2;
  }
  if (N == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    std::vector<double> hd(N), he(N, 0.0);
    CK(cudaMemcpyAsync(hd.data(), d, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(he.data(), e, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double *dw = buf<double>(c, "w_out", N);
    std::vector<Problem> pr;
    long long o = 0, oz = 0;
    for (int p = 0; p < nprob; ++p) {
      if (n[p] > 0)
        pr.push_back(Problem{n[p], hd.data() + o, he.data() + o, z + oz, n[p], dw + o});
      o += n[p];
      oz += (long long)n[p] * n[p];
    }
    int info = solve_core(c, pr, st);
    CK(cudaMemcpyAsync(d, dw, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    return info;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_mdsbevd_dev(int n, int kd, const double *ab, int ldab, double *w, double *z, int ldz,
                    void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -1;
  if (kd < 0) {
    c.err = "hss_mdsbevd_dev: kd < 0";
    return -2;
  }
  if (ldab < kd + 1) return -4;
  if (ldz < std::max(1, n)) return -7;
  if (n == 0) return 0;
  try {
    return band_solve(c, n, kd, ab, ldab, z, ldz, w, (cudaStream_t)stream);
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_mdbdsdc_dev(int n, double *d, double *e, double *u, int ldu, double *vt, int ldvt,
                    void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -1;
  if (ldu < std::max(1, n)) return -5;
  if (ldvt < std::max(1, n)) return -7;
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    std::vector<double> hd(n), he(std::max(n, 1), 0.0);
    CK(cudaMemcpyAsync(hd.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (n > 1) CK(cudaMemcpyAsync(he.data(), e, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double *dw = buf<double>(c, "w_out", n);
    const int info = svd_solve(c, false, n, hd, he, u, ldu, vt, ldvt, dw, true, st);
    CK(cudaMemcpyAsync(d, dw, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    return info;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

void mdbdsdc_(const char *uplo, const char *compq, const int *n_, double *d, double *e, double *u,
              const int *ldu_, double *vt, const int *ldvt_, double *q, int *iq, double *work,
              int *iwork, int *info, size_t, size_t) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  (void)q; (void)iq; (void)work; (void)iwork;
  const int n = *n_, ldu = *ldu_, ldvt = *ldvt_;
  const char cu = uplo[0], cq = compq[0];
  const int iuplo = (cu == 'U' || cu == 'u') ? 1 : (cu == 'L' || cu == 'l') ? 2 : 0;
  const int icompq = (cq == 'N' || cq == 'n') ? 0 : (cq == 'P' || cq == 'p') ? 1 : (cq == 'I' || cq == 'i') ? 2 : -1;
  *info = 0;  // argument numbering as SRC/mdbdsdc.f90 (DBDSDC)
  if (iuplo == 0) *info = -1;
  else if (icompq < 0) *info = -2;
  else if (n < 0) *info = -3;
  else if (ldu < 1 || (icompq == 2 && ldu < n)) *info = -7;
  else if (ldvt < 1 || (icompq == 2 && ldvt < n)) *info = -9;
  if (*info == 0 && icompq == 1) {  // the compact form (DLASDA) is not built
    *info = -2;
    c.err = "MDBDSDC: COMPQ = 'P' (compact singular vectors) is not supported";
    return;
  }
  if (*info != 0) {
    c.err = "MDBDSDC: illegal argument " + std::to_string(-*info);
    return;
  }
  if (n == 0) return;
  if (n == 1) {  // mdbdsdc.f90: U = sign(d), VT = 1, d = |d|
    if (icompq == 2) { u[0] = d[0] < 0.0 ? -1.0 : 1.0; vt[0] = 1.0; }
    d[0] = std::fabs(d[0]);
    return;
  }
  try {
    cudaStream_t st = nullptr;
    std::vector<double> hd(d, d + n), he(e, e + (n - 1));
    const bool vec = icompq == 2;
    double *dU = buf<double>(c, "z_out", vec ? (size_t)n * n : 1);
    double *dVT = buf<double>(c, "vt_out", vec ? (size_t)n * n : 1);
    double *dw = buf<double>(c, "w_out", n);
    *info = svd_solve(c, iuplo == 2, n, hd, he, dU, n, dVT, n, dw, vec, st);
    if (vec) {
      CK(cudaMemcpy2DAsync(u, sizeof(double) * ldu, dU, sizeof(double) * n, sizeof(double) * n, n,
                           cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpy2DAsync(vt, sizeof(double) * ldvt, dVT, sizeof(double) * n, sizeof(double) * n,
                           n, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaMemcpyAsync(d, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int i = 0; i + 1 < n; ++i) e[i] = 0.0;  // E is destroyed, as in the reference
  } catch (CudaError &ex) {
    c.err = ex.msg;
    *info = 1000000;
  }
}

// MDBDSVD (SRC/mdbdsvd.f90:1) on device arrays.  The band's leaves are at most
// 64 rows and 96 columns, so sb <= 32.
int hss_mdbdsvd_dev(int n, int sb, const double *ab, int ldab, double *s, double *u, int ldu,
                    double *vt, int ldvt, int smlsiz, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -1;
  if (sb < 1 || sb > n || sb > 32) {
    c.err = "hss_mdbdsvd_dev: sb must be in 1 .. min(n, 32)";
    return -2;
  }
  if (ldab < sb + 1) return -4;
  if (ldu < std::max(1, n)) return -7;
  if (ldvt < std::max(1, n)) return -9;
  if (smlsiz < 3) return -10;
  if (n == 0) return 0;
  try {
    return bsvd_core(c, n, sb, ab, ldab, std::max(smlsiz, 3 * sb), u, ldu, vt, ldvt, s,
                     (cudaStream_t)stream);
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    return 1000001;
  }
}

// MDBDSVD(N, SB, AB, LDAB, A, S, U, LDU, VT, LDVT, SMLSIZ, WORK, LWORK, IWORK,
// INFO) with host arrays.  Argument checks as mdbdsvd.f90:120-137 (the second
// group overrides the first), plus LDAB >= SB + 1 (-4) and SB <= 32 (-3).  A,
// WORK, LWORK and IWORK are not used (the reference's workspaces); SMLSIZ is
// raised to 3 SB as MDBDSVDT does.
void mdbdsvd_(const int *n_, const int *sb_, double *ab, const int *ldab_, double *a, double *s,
              double *u, const int *ldu_, double *vt, const int *ldvt_, int *smlsiz_, double *work,
              int *lwork_, int *iwork, int *info) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  (void)a; (void)work; (void)lwork_; (void)iwork;
  const int n = *n_, sb = *sb_, ldab = *ldab_, ldu = *ldu_, ldvt = *ldvt_;
  *info = 0;
  if (n < 0 || n < sb) *info = -2;
  else if (sb < 1) *info = -3;
  if (ldu < n) *info = -9;
  else if (ldvt < n) *info = -10;
  else if (*smlsiz_ < 3) *info = -11;
  if (*info == 0 && ldab < sb + 1) *info = -4;
  if (*info == 0 && sb > 32) {
    *info = -3;
    c.err = "MDBDSVD: semibandwidths above 32 are not supported";
    return;
  }
  if (*info != 0) {
    c.err = "MDBDSVD: illegal argument " + std::to_string(-*info);
    return;
  }
  if (n > *smlsiz_ && *smlsiz_ < 3 * sb) *smlsiz_ = 3 * sb;
  if (n == 0) return;
  try {
    cudaStream_t st = nullptr;
    const long long lda = sb + 1;
    std::vector<double> hb((size_t)lda * n);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i <= sb; ++i) hb[(size_t)j * lda + i] = ab[(size_t)j * ldab + i];  // AB(SB+1+I-J, J)
    double *dab = buf<double>(c, "band_ab", hb.size());
    double *dU = buf<double>(c, "z_out", (size_t)n * n);
    double *dVT = buf<double>(c, "vt_out", (size_t)n * n);
    double *dw = buf<double>(c, "w_out", n);
    CK(cudaMemcpyAsync(dab, hb.data(), sizeof(double) * hb.size(), cudaMemcpyHostToDevice, st));
    *info = bsvd_core(c, n, sb, dab, lda, std::max(*smlsiz_, 3 * sb), dU, n, dVT, n, dw, st);
    if (*info != 0) return;
    CK(cudaMemcpy2DAsync(u, sizeof(double) * ldu, dU, sizeof(double) * n, sizeof(double) * n, n,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpy2DAsync(vt, sizeof(double) * ldvt, dVT, sizeof(double) * n, sizeof(double) * n, n,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(s, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c.stats.host_h2d_bytes = 8LL * lda * n;
    c.stats.host_d2h_bytes = 16LL * n * n + 8LL * n;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    *info = 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    *info = 1000001;
  }
}

// Host band arrays -> device upper storage (lower storage converted), then the
// device solve; results copied back.  Shared by MDSBEVD and MDSBEDC.
static int band_host(Ctx &c, bool lower, int n, int kd, const double *ab, int ldab, double *w,
                     double *z, int ldz, bool wantz) {
  cudaStream_t st = nullptr;
  const long long ldu = kd + 1;
  std::vector<double> hu((size_t)ldu * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - kd); i <= j; ++i)
      hu[(size_t)j * ldu + kd + i - j] =
          lower ? ab[(size_t)i * ldab + (j - i)] : ab[(size_t)j * ldab + kd + i - j];
  double *dab = buf<double>(c, "band_ab", hu.size());
  double *dz = buf<double>(c, "z_out", (size_t)n * n);
  double *dw = buf<double>(c, "w_out", n);
  CK(cudaMemcpyAsync(dab, hu.data(), sizeof(double) * hu.size(), cudaMemcpyHostToDevice, st));
  const int info = band_solve(c, n, kd, dab, ldu, dz, n, dw, st, wantz);
  if (wantz)
    CK(cudaMemcpy2DAsync(z, sizeof(double) * ldz, dz, sizeof(double) * n, sizeof(double) * n, n,
                         cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(w, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return info;
}

void mdsbevd_(const char *compz, const char *uplo, const int *n_, const int *kd_, double *ab,
              const int *ldab_, double *d, double *q, const int *ldq_, double *work,
              const int *lwork_, int *iwork, const int *liwork_, int *info, size_t, size_t) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  const int n = *n_, kd = *kd_, ldab = *ldab_, ldq = *ldq_, lwork = *lwork_, liwork = *liwork_;
  const char cz = compz[0];
  const int icompz = (cz == 'N' || cz == 'n') ? 0 : (cz == 'I' || cz == 'i') ? 2 : -1;
  const bool lquery = (lwork == -1 || liwork == -1);
  *info = 0;
  // argument numbering as SRC/mdsbevd.f90:228-263
  if (icompz < 0) *info = -1;
  else if (n < 0) *info = -2;
  else if (ldq < 1 || (icompz > 0 && ldq < std::max(1, n))) *info = -6;
  long long lwmin = 1, liwmin = 1;
  if (*info == 0) {
    const int smlsiz = 25;  // ILAENV(9, 'DSTEDC') as the reference (mdsbevd.f90:255)
    if (n <= 1 || icompz == 0) { lwmin = 1; liwmin = 1; }
    else if (n <= smlsiz) { lwmin = 2LL * (n - 1); liwmin = 1; }
    else { lwmin = 1 + 4LL * n + (long long)n * n; liwmin = 3 + 5LL * n; }
    if (work) work[0] = (double)lwmin;
    if (iwork) iwork[0] = (int)std::min<long long>(liwmin, 2147483647LL);
    if (lwork < lwmin && !lquery) *info = -8;
    else if (liwork < liwmin && !lquery) *info = -10;
  }
  if (*info == 0 && (kd < 0 || ldab < kd + 1)) *info = -4;
  if (*info != 0) {
    c.err = "MDSBEVD: illegal argument " + std::to_string(-*info);
    return;
  }
  if (lquery || n == 0) return;
  if (n == 1) {
    d[0] = ab[kd];
    if (icompz != 0) q[0] = 1.0;
    return;
  }
  (void)uplo;  // the reference reads the upper band whatever UPLO says
  try {
    *info = band_host(c, false, n, kd, ab, ldab, d, q, ldq, icompz != 0);
    if (work) work[0] = (double)lwmin;
    if (iwork) iwork[0] = (int)std::min<long long>(liwmin, 2147483647LL);
  } catch (CudaError &ex) {
    c.err = ex.msg;
    *info = 1000000;
  }
}

void mdsbedc_(const char *jobz, const char *uplo, const int *n_, const int *kd_, double *ab,
              const int *ldab_, double *w, double *z, const int *ldz_, double *work,
              const int *lwork_, int *iwork, const int *liwork_, int *info, size_t, size_t) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  const int n = *n_, kd = *kd_, ldab = *ldab_, ldz = *ldz_, lwork = *lwork_, liwork = *liwork_;
  const bool wantz = jobz[0] == 'V' || jobz[0] == 'v';
  const bool lower = uplo[0] == 'L' || uplo[0] == 'l';
  const bool lquery = (lwork == -1 || liwork == -1);
  long long lwmin = 1, liwmin = 1;
  if (n > 1) {  // SRC/mdsbedc.f90:190-201
    if (wantz) { liwmin = 3 + 5LL * n; lwmin = 1 + 5LL * n + 2LL * n * n; }
    else { liwmin = 1; lwmin = 2LL * n; }
  }
  *info = 0;
  if (!(wantz || jobz[0] == 'N' || jobz[0] == 'n')) *info = -1;
  else if (!(lower || uplo[0] == 'U' || uplo[0] == 'u')) *info = -2;
  else if (n < 0) *info = -3;
  else if (kd < 0) *info = -4;
  else if (ldab < kd + 1) *info = -6;
  else if (ldz < 1 || (wantz && ldz < n)) *info = -9;
  if (*info == 0) {
    if (work) work[0] = (double)lwmin;
    if (iwork) iwork[0] = (int)std::min<long long>(liwmin, 2147483647LL);
    if (lwork < lwmin && !lquery) *info = -11;
    else if (liwork < liwmin && !lquery) *info = -13;
  }
  if (*info != 0) {
    c.err = "MDSBEDC: illegal argument " + std::to_string(-*info);
    return;
  }
  if (lquery || n == 0) return;
  if (n == 1) {
    w[0] = lower ? ab[0] : ab[kd];
    if (wantz) z[0] = 1.0;
    return;
  }
  try {
    *info = band_host(c, lower, n, kd, ab, ldab, w, z, ldz, wantz);
  } catch (CudaError &ex) {
    c.err = ex.msg;
    *info = 1000000;
  }
}

void mdstedc_(const char *compz, const int *n_, double *d, double *e, double *z, const int *ldz_,
              double *work, const int *lwork_, int *iwork, const int *liwork_, int *info,
              size_t /*compz_len*/) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  const int n = *n_, ldz = *ldz_, lwork = *lwork_, liwork = *liwork_;
  const char cz = compz[0];
  int icompz = (cz == 'N' || cz == 'n') ? 0 : (cz == 'V' || cz == 'v') ? 1 : (cz == 'I' || cz == 'i') ? 2 : -1;
  *info = 0;
  const bool lquery = (lwork == -1 || liwork == -1);
  if (icompz < 0) *info = -1;
  else if (n < 0) *info = -2;
  else if (ldz < 1 || (icompz > 0 && ldz < std::max(1, n))) *info = -6;
  long long lwmin = 1, liwmin = 1;
  if (*info == 0) {
    // the reference's workspace formulas (SRC/mdstedc.f90:211-229), with its
    // SMLSIZ = ILAENV(9, 'DSTEDC') = 25 (the GPU's own leaf size is separate)
    const int smlsiz = 25;
    if (n <= 1 || icompz == 0) { lwmin = 1; liwmin = 1; }
    else if (n <= smlsiz) { lwmin = 2LL * (n - 1); liwmin = 1; }
    else if (icompz == 1) {
      int lgn = 0;
      while ((1LL << lgn) < n) ++lgn;  // ceil(log2 n), as LGN there
      lwmin = 1 + 3LL * n + 2LL * n * lgn + 4LL * n * n;
      liwmin = 6 + 6LL * n + 5LL * n * lgn;
    } else { lwmin = 1 + 4LL * n + (long long)n * n; liwmin = 3 + 5LL * n; }
    if (work) work[0] = (double)lwmin;
    if (iwork) iwork[0] = (int)std::min<long long>(liwmin, 2147483647LL);
    if (lwork < lwmin && !lquery) *info = -8;
    else if (liwork < liwmin && !lquery) *info = -10;
  }
  if (*info != 0) {
    c.err = "MDSTEDC: illegal argument " + std::to_string(-*info);
    return;
  }
  if (lquery || n == 0) return;
  if (n == 1) {
    if (icompz != 0) z[0] = 1.0;
    return;
  }
  try {
    cudaStream_t st = nullptr;
    std::vector<double> hd(d, d + n), he(e, e + (n - 1));
    double *dz = buf<double>(c, "z_out", (size_t)n * n);
    double *dw = buf<double>(c, "w_out", n);
    if (icompz == 0) {
      // eigenvalues only: the same solve, vectors discarded (the reference
      // calls DSTERF here, mdstedc.f90:264-267)
      *info = mdstedc_core(c, n, hd, he, dz, n, dw, st);
    } else if (icompz == 1) {
      // Z holds Q0 on entry: copied in, multiplied on the device, copied out
      CK(cudaMemcpy2DAsync(dz, sizeof(double) * n, z, sizeof(double) * ldz, sizeof(double) * n, n,
                           cudaMemcpyHostToDevice, st));
      *info = mdstedc_v_core(c, n, hd, he, dz, n, dw, st);
      if (*info == 0)
        CK(cudaMemcpy2DAsync(z, sizeof(double) * ldz, dz, sizeof(double) * n, sizeof(double) * n,
                             n, cudaMemcpyDeviceToHost, st));
      c.stats.host_d2h_bytes = 8LL * n * n;
    } else {
      // large problems: Z is zeroed on host threads while the GPU solves, and
      // only the columns' supported rows come back (unless they fill Z)
      HostFill fill(z, n, ldz, n >= 2048);
      PackedZ pz;
      pz.want = fill.active();
      {
        PzScope scope(c, &pz);
        *info = mdstedc_core(c, n, hd, he, dz, n, dw, st);
      }
      if (pz.packed) {
        double *hz = zstage(c, (size_t)std::max<long long>(pz.total, 1));
        CK(cudaMemcpyAsync(hz, pz.dbuf, sizeof(double) * pz.total, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        fill.finish(&pz, hz);  // each worker fills in its columns once they are zeroed
        // packed rows plus the slot and row-range tables read on the host
        c.stats.host_d2h_bytes = 8LL * pz.total + 12LL * n;
      } else {
        fill.finish(nullptr, nullptr);
        CK(cudaMemcpy2DAsync(z, sizeof(double) * ldz, dz, sizeof(double) * n, sizeof(double) * n, n,
                             cudaMemcpyDeviceToHost, st));
        c.stats.host_d2h_bytes = 8LL * n * n;
      }
    }
    CK(cudaMemcpyAsync(d, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c.stats.host_d2h_bytes += 8LL * n;
    c.stats.host_h2d_bytes = 16LL * n + (icompz == 1 ? 8LL * n * n : 0LL);
    if (work) work[0] = (double)lwmin;
    if (iwork) iwork[0] = (int)std::min<long long>(liwmin, 2147483647LL);
  } catch (CudaError &ex) {
    c.err = ex.msg;
    *info = 1000000;
  }
}

int hss_secular_dev(int k, const double *dlamda, const double *z, double rho, double *lam,
                    double *difl, double *difr, int *iters, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (k <= 0) return k < 0 ? -1 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    std::vector<int> s(1, 0), K(1, k), off{0, k};
    std::vector<double> r(1, rho);
    int *vs = buf<int>(c, "x_s", 1), *vK = buf<int>(c, "x_K", 1), *vo = buf<int>(c, "x_off", 2);
    double *vr = buf<double>(c, "x_rho", 1);
    int *status = buf<int>(c, "x_status", 1);
    h2d(vs, s, st); h2d(vK, K, st); h2d(vo, off, st); h2d(vr, r, st);
    CK(cudaMemsetAsync(status, 0, sizeof(int), st));
    LevelView lv{vs, vK, vr, vo, 1};
    float *guess = nullptr;
    if (c.cfg.predictor >= 2) {  // (3 runs the plain pre-solve here)
      guess = buf<float>(c, "x_guess", k);
      launch_secular_guess32(lv, k, k, k, dlamda, z, buf<float>(c, "x_d32", k),
                             buf<float>(c, "x_z32", k), guess, st);
    } else if (c.cfg.predictor && c.pred_ready) {
      float *feat = buf<float>(c, "x_feat", (size_t)k * (mlp_nfeat() + 1));
      guess = buf<float>(c, "x_guess", k);
      launch_secular_mid(lv, k, k, dlamda, z, feat, st);
      launch_predict(k, feat, buf<char>(c, "pred_wb", 0), buf<float>(c, "pred_norm", 0), guess, st);
    }
    unsigned long long *cnt = (unsigned long long *)buf<char>(c, "x_counts", 24);
    CK(cudaMemsetAsync(cnt, 0, 24, st));
    launch_secular(lv, k, k, dlamda, z, lam, difl, difr, iters, status, cnt, guess, st, false,
                   c.cfg.predictor >= 2);
    unsigned long long hc[2];
    CK(cudaMemcpyAsync(hc, cnt, 16, cudaMemcpyDeviceToHost, st));
    int hs = 0;
    CK(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    c.stats.secular_iters = (long long)hc[0];
    c.stats.secular_roots = k;
    c.stats.predictor_fallbacks = (long long)hc[1];
    return hs ? 1 : 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_lowner_dev(int k, const double *dlamda, const double *difl, const double *difr, double *z,
                   double *alpha, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (k <= 0) return k < 0 ? -1 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    std::vector<int> s(1, 0), K(1, k), off{0, k};
    std::vector<double> r(1, 1.0);
    int *vs = buf<int>(c, "x_s", 1), *vK = buf<int>(c, "x_K", 1), *vo = buf<int>(c, "x_off", 2);
    double *vr = buf<double>(c, "x_rho", 1);
    h2d(vs, s, st); h2d(vK, K, st); h2d(vo, off, st); h2d(vr, r, st);
    LevelView lv{vs, vK, vr, vo, 1};
    double *zh = buf<double>(c, "x_zhat", k);
    launch_lowner(lv, k, dlamda, difl, difr, z, zh, st);
    launch_alpha(lv, k, dlamda, difl, difr, zh, alpha, st);
    CK(cudaMemcpyAsync(z, zh, sizeof(double) * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_cauchy_eig_dev(int k, const double *F, const double *u, const double *v,
                       const double *difl, const double *difr, double *C, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (k < 0) return -1;
  try {
    launch_cauchy_eig(k, F, u, v, difl, difr, C, (cudaStream_t)stream);
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_dhssevc_dev(int k, int ni, double tol, const double *F, const double *u, const double *v,
                    const double *difl, const double *difr, double *Q, int ldq, int nrows,
                    void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (k < 0) return -1;
  if (ni < 1) return -2;
  if (ldq < std::max(1, nrows)) return -10;
  if (k == 0 || nrows == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    int rank = 0;
    float t2[2] = {0.f, 0.f};
    hss_dhssevc_core(k, ni, tol, c.cfg.precision, F, u, v, difl, difr, Q, ldq, nrows, &rank, st,
                     t2);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    c.stats.max_rank = rank;
    // construction and product times of this call (CUDA events)
    c.stats.stage_ms[HSS_ST_HSS_BUILD] = t2[0];
    c.stats.stage_ms[HSS_ST_HSS_MM] = t2[1];
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    return 1000001;
  }
}

int hss_cauchyhssmm_dev(int n, const double *D, const double *F, const double *u, const double *v,
                        int ni, double tol, double *B, int ldb, int ncb, float *times,
                        void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -1;
  if (ni < 1) return -6;
  if (ldb < std::max(1, n)) return -9;
  if (ncb < 0) return -10;
  if (n == 0 || ncb == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    int rank = 0;
    hss_cauchyhssmm_core(n, D, F, u, v, ni, tol, c.cfg.precision, B, ldb, ncb, &rank, times, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    c.stats.max_rank = rank;
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    return 1000001;
  }
}

void cauchyhssmm_(const double *D, const double *F, const double *U, const double *V, const int *n_,
                  const int *ni_, const double *tol_, const int *ncol_, double *B, const int *ldb_,
                  double *time) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  const int n = *n_, ni = *ni_, ldb = *ldb_;
  (void)ncol_;  // the GPU multiply takes all columns of B in one pass
  if (n <= 0 || ni < 1 || ldb < n) {
    c.err = "CauchyHssMM: bad N, ni or LDB";
    if (time) { time[0] = 0.0; time[1] = 0.0; }
    return;
  }
  try {
    cudaStream_t st = nullptr;
    double *dv = buf<double>(c, "chm_in", 4 * (size_t)n);
    double *dB = buf<double>(c, "chm_B", (size_t)n * n);
    CK(cudaMemcpyAsync(dv, D, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dv + n, F, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dv + 2 * n, U, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dv + 3 * n, V, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpy2DAsync(dB, sizeof(double) * n, B, sizeof(double) * ldb, sizeof(double) * n, n,
                         cudaMemcpyHostToDevice, st));
    int rank = 0;
    float t[2] = {0.f, 0.f};
    hss_cauchyhssmm_core(n, dv, dv + n, dv + 2 * n, dv + 3 * n, ni, *tol_, c.cfg.precision, dB, n,
                         n, &rank, t, st);
    CK(cudaMemcpy2DAsync(B, sizeof(double) * ldb, dB, sizeof(double) * n, sizeof(double) * n, n,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c.stats.max_rank = rank;
    if (time) { time[0] = 1e-3 * t[0]; time[1] = 1e-3 * t[1]; }
  } catch (CudaError &ex) {
    c.err = ex.msg;
  } catch (HssError &ex) {
    c.err = ex.msg;
  }
}

// SvdHssUpdat (SRC/SvdHssUpdat.f90:1) on device arrays.
int hss_svdhssupdat_dev(int n, double *d, double *f, double *z, double *vt, int ldvt, double tol,
                        int ni, int *k, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (k) *k = 0;
  if (n < 0) return -1;
  if (ldvt < std::max(1, n)) return -6;
  if (ni < 1) return -8;
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    memset(&c.stats, 0, sizeof c.stats);
    int *status = buf<int>(c, "su_status", 8);
    CK(cudaMemsetAsync(status, 0, 8 * sizeof(int), st));
    int rank = 0;
    float t2[2] = {0.f, 0.f};
    const int K = svd_update_core(n, d, f, z, vt, ldvt, tol, ni, c.cfg.precision, &rank, status,
                                  t2, st);
    int hst[8];
    CK(cudaMemcpyAsync(hst, status, sizeof hst, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    if (k) *k = K;
    c.stats.max_rank = rank;
    c.stats.total_k = K;
    c.stats.secular_roots = K;
    c.stats.secular_iters = (long long)(((unsigned long long)(unsigned)hst[3] << 32) | (unsigned)hst[2]);
    c.stats.stage_ms[HSS_ST_HSS_BUILD] = t2[0];
    c.stats.stage_ms[HSS_ST_HSS_MM] = t2[1];
    return hst[0] ? hst[0] : 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    return 1000001;
  }
}

// SvdHssUpdat(D,F,Z,V,N0,TOL,ni) with host arrays (V: N0 x N0, leading dimension
// N0, rows = right singular vectors).  The reference has no INFO argument:
// failures leave the outputs untouched and set hss_last_error().
void svdhssupdat_(double *D, double *F, double *Z, double *V, const int *n0_, const double *tol_,
                  const int *ni_) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  const int n = *n0_, ni = *ni_;
  c.err.clear();  // without INFO, an empty hss_last_error() reports success
  if (n <= 0 || ni < 1) {
    c.err = "SvdHssUpdat: bad N0 or ni";
    return;
  }
  try {
    cudaStream_t st = nullptr;
    double *dv = buf<double>(c, "su_in", 3 * (size_t)n);
    double *dV = buf<double>(c, "su_V", (size_t)n * n);
    CK(cudaMemcpyAsync(dv + n, F, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dv + 2 * n, Z, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dV, V, sizeof(double) * n * n, cudaMemcpyHostToDevice, st));
    int k = 0;
    const int info = hss_svdhssupdat_dev(n, dv, dv + n, dv + 2 * n, dV, n, *tol_, ni, &k, st);
    if (info != 0) {
      if (info < 1000000) c.err = "SvdHssUpdat: a secular root did not converge";
      return;
    }
    CK(cudaMemcpyAsync(D, dv, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(F, dv + n, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(Z, dv + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(V, dV, sizeof(double) * n * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c.stats.host_h2d_bytes = 8LL * n * (n + 2);
    c.stats.host_d2h_bytes = 8LL * n * (n + 3);
  } catch (CudaError &ex) {
    c.err = ex.msg;
  } catch (HssError &ex) {
    c.err = ex.msg;
  }
}

// ------------------------------------------------------- HSS Cholesky ----
struct hss_chol {
  CholFactor F;
};

int hss_chol_factor_dev(int n, const double *A, int lda, int ni, double tol, int prank, int ps,
                        hss_chol **out, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (out) *out = nullptr;
  if (n < 1) return -1;
  if (lda < n) return -3;
  if (ni < 1 || ni > CH_MAXM) return -4;
  if (prank < 1) return -6;
  if (ps < 0) return -7;
  if (!out) return -8;
  cudaStream_t st = (cudaStream_t)stream;
  hss_chol *h = new (std::nothrow) hss_chol;
  if (!h) return -8;
  try {
    memset(&c.stats, 0, sizeof c.stats);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, st));
    const int info = hss_chol_factor_core(n, A, lda, ni, tol, prank, ps, 0x5eedull, h->F, st);
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c.stats.ms_total = ms;
    c.stats.max_rank = h->F.max_rank;
    c.stats.n_levels = (int)h->F.lv.size();
    if (info != 0) {
      c.err = info == 1 ? "HSS Cholesky: a diagonal block is not positive definite"
                        : "HSS Cholesky: a node has more than 128 rows";
      delete h;
      return info;
    }
    *out = h;
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    delete h;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    delete h;
    return 1000001;
  }
}

int hss_chol_solve_dev(const hss_chol *f, double *B, int ldb, int nrhs, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (!f) return -1;
  if (ldb < f->F.n) return -3;
  if (nrhs < 0) return -4;
  if (nrhs == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    hss_chol_solve_core(f->F, B, ldb, nrhs, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    return 1000001;
  }
}

int hss_chol_pcg_dev(const hss_chol *f, int n, const double *A, int lda, const double *b,
                     double *x, double tau, int maxit, int *iters, double *relres, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 1) return -2;
  if (f && f->F.n != n) return -2;
  if (lda < n) return -4;
  if (maxit < 0) return -8;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    double rr = 0.0;
    const int it = hss_chol_pcg_core(f ? &f->F : nullptr, n, A, lda, b, x, tau, maxit, &rr, st);
    CK(cudaGetLastError());
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    return 1000001;
  }
}

int hss_chol_info(const hss_chol *f, int *n, int *max_rank, int *levels, int *root,
                  long long *bytes) {
  if (!f) return -1;
  if (n) *n = f->F.n;
  if (max_rank) *max_rank = f->F.max_rank;
  if (levels) *levels = (int)f->F.lv.size();
  if (root) *root = f->F.Nroot;
  if (bytes) *bytes = f->F.fac_bytes;
  return 0;
}

void hss_chol_free(hss_chol *f) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  delete f;
}

// HssCholSolver(RS,WPCG,A,LDA,b,ni,tol,prank,pp,tau,MaxIt,info) with host
// arrays: N = LDA (as the reference); b (N) is replaced by the solution.
void hsscholsolver_(const char *rs, const char *wpcg, double *A, const int *lda_, double *b,
                    const int *ni_, const double *tol_, const int *prank_, const int *pp_,
                    const double *tau_, const int *maxit_, int *info, size_t rs_len,
                    size_t wpcg_len) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  *info = 0;
  (void)rs_len;
  (void)wpcg_len;
  const char r = (char)toupper((unsigned char)rs[0]), w = (char)toupper((unsigned char)wpcg[0]);
  if (r != 'R' && r != 'S') { *info = -1; return; }
  if (w != 'Y' && w != 'N') { *info = -2; return; }
  const int n = *lda_, ni = *ni_, prank = *prank_, pp = *pp_;
  if (n < 1) { *info = -4; return; }
  if (ni < 1 || ni > CH_MAXM) { *info = -6; return; }
  if (prank < 1) { *info = -8; return; }
  if (r == 'R' && pp < 0) { *info = -9; return; }
  if (*maxit_ < 0) { *info = -11; return; }
  try {
    cudaStream_t st = nullptr;
    double *dA = buf<double>(c, "hc_hostA", (size_t)n * n);
    double *dv = buf<double>(c, "hc_hostv", 2 * (size_t)n);
    CK(cudaMemcpyAsync(dA, A, sizeof(double) * n * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dv, b, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    hss_chol *f = nullptr;
    const int ps = r == 'R' ? prank + pp : 0;
    const int fi = hss_chol_factor_dev(n, dA, n, ni, *tol_, prank, ps, &f, st);
    if (fi != 0) { *info = fi; return; }
    if (w == 'N') {
      const int si = hss_chol_solve_dev(f, dv, n, 1, st);
      if (si != 0) { *info = si; hss_chol_free(f); return; }
      CK(cudaMemcpyAsync(b, dv, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    } else {
      int it = 0;
      double rr = 0.0;
      const int pi = hss_chol_pcg_dev(f, n, dA, n, dv, dv + n, *tau_, *maxit_, &it, &rr, st);
      if (pi != 0) { *info = pi; hss_chol_free(f); return; }
      CK(cudaMemcpyAsync(b, dv + n, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
      c.stats.secular_iters = it;  // the CG steps taken
    }
    CK(cudaStreamSynchronize(st));
    hss_chol_free(f);
    c.stats.host_h2d_bytes = 8LL * n * (n + 1);
    c.stats.host_d2h_bytes = 8LL * n;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    *info = 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    *info = 1000001;
  }
}

// MDLASD20's deflation alone (host code, no GPU): for the CPU tests.
int hss_svdupd_deflate(int n, double *f, double *z, int *idxp, int *nrot) {
  if (n < 0) return -1;
  const SvdUpdDeflation df = svdupd_deflate(n, f, z);
  for (int j = 0; j < n; ++j) idxp[j] = df.idxp[j];
  if (nrot) *nrot = (int)df.rot.size();
  return df.K;
}

int hss_bsvd_tree(int n, int sb, int smlsiz, int *leaf_start, int *leaf_rows, int *leaf_cols,
                  int *nleaves) {
  if (n < 1 || sb < 1 || sb > 32 || sb > n || smlsiz < 3) return -1;
  std::vector<std::vector<BNode>> lv;
  const int depth = bsvd_tree(n, sb, std::max(smlsiz, 3 * sb), lv);
  if (depth < 0) return -2;
  const std::vector<BNode> &leaves = lv.back();
  for (size_t i = 0; i < leaves.size(); ++i) {
    leaf_start[i] = leaves[i].s;
    leaf_rows[i] = leaves[i].X;
    leaf_cols[i] = leaves[i].X + leaves[i].sq;
  }
  *nleaves = (int)leaves.size();
  return depth;
}

int hss_rcp_dev(int n, const double *x, double *y, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -1;
  try {
    launch_rcp(n, x, y, (cudaStream_t)stream);
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_dhssmm_dev(int n, const double *A, int lda, double *B, int ldb, int k, double tol, int ni,
                   int side, float *times, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -1;
  if (lda < std::max(1, n)) return -3;
  if (ldb < std::max(1, side == 0 ? n : k)) return -5;
  if (k < 0) return -6;
  if (ni < 1) return -8;
  if (side != 0 && side != 1) return -9;
  if (n == 0 || k == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  try {
    int rank = 0;
    hss_dhssmm_core(n, A, lda, B, ldb, k, tol, ni, side, c.cfg.precision, &rank, times, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    c.stats.max_rank = rank;
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    return 1000001;
  }
}

// DHSSMM (side 0) and DHSSMML (side 1) with host arrays.  INFO numbering
// follows the argument list A,LDA,M,N,B,LDB,K,tol,prank,ni,ncol,time,info.
static void dhssmm_host(int side, const double *A, int lda, int m, int n, double *B, int ldb,
                        int k, double tol, int ni, int ncol, double *time, int *info) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  *info = 0;
  if (n < 0) *info = -4;
  else if (m != n) *info = -3;
  else if (lda < std::max(1, n)) *info = -2;
  else if (ldb < std::max(1, side == 0 ? n : k)) *info = -6;
  else if (k < 0) *info = -7;
  else if (ni < 1) *info = -10;
  else if (ncol < 1) *info = -11;
  if (time) { time[0] = 0.0; time[1] = 0.0; }
  if (*info != 0) {
    c.err = side == 0 ? "DHSSMM: bad argument" : "DHSSMML: bad argument";
    return;
  }
  if (n == 0 || k == 0) return;
  try {
    cudaStream_t st = nullptr;
    const int br = side == 0 ? n : k, bc = side == 0 ? k : n;
    double *dA = buf<double>(c, "hm_A", (size_t)n * n);
    double *dB = buf<double>(c, "hm_B", (size_t)br * bc);
    CK(cudaMemcpy2DAsync(dA, sizeof(double) * n, A, sizeof(double) * lda, sizeof(double) * n, n,
                         cudaMemcpyHostToDevice, st));
    CK(cudaMemcpy2DAsync(dB, sizeof(double) * br, B, sizeof(double) * ldb, sizeof(double) * br, bc,
                         cudaMemcpyHostToDevice, st));
    int rank = 0;
    float t[2] = {0.f, 0.f};
    hss_dhssmm_core(n, dA, n, dB, br, k, tol, ni, side, c.cfg.precision, &rank, t, st);
    CK(cudaMemcpy2DAsync(B, sizeof(double) * ldb, dB, sizeof(double) * br, sizeof(double) * br, bc,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c.stats.max_rank = rank;
    if (time) { time[0] = 1e-3 * t[0]; time[1] = 1e-3 * t[1]; }
  } catch (CudaError &ex) {
    c.err = ex.msg;
    *info = 1000000;
  } catch (HssError &ex) {
    c.err = ex.msg;
    *info = 1000001;
  }
}

void dhssmm_(const double *A, const int *lda, const int *m, const int *n, double *B, const int *ldb,
             const int *k, const double *tol, const int *prank, const int *ni, const int *ncol,
             double *time, int *info) {
  (void)prank;  // declared but not read by the reference's construction
  dhssmm_host(0, A, *lda, *m, *n, B, *ldb, *k, *tol, *ni, *ncol, time, info);
}

void dhssmml_(const double *A, const int *lda, const int *m, const int *n, double *B, const int *ldb,
              const int *k, const double *tol, const int *prank, const int *ni, const int *ncol,
              double *time, int *info) {
  (void)prank;
  dhssmm_host(1, A, *lda, *m, *n, B, *ldb, *k, *tol, *ni, *ncol, time, info);
}

int hss_gemm_dev(int m, int n, int k, const double *A, int lda, const double *B, int ldb,
                 double *C, int ldc, int beta, int precision, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (k < 0) return -3;
  if (lda < std::max(1, m)) return -5;
  if (ldb < std::max(1, k)) return -7;
  if (ldc < std::max(1, m)) return -9;
  if (precision < 0 || precision > 1) return -11;
  if (m == 0 || n == 0) return 0;
  try {
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<GemmDesc> p{{A, B, C, lda, ldb, ldc, m, n, k, beta ? 1 : 0, 0}};
    int *err = buf<int>(c, "gemm_err", 1);
    CK(cudaMemsetAsync(err, 0, sizeof(int), st));
    launch_gemm(p, precision, st);
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    if (herr) {
      c.err = "tensor-core GEMM: bounded wait timed out";
      return 1;
    }
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_predictor_nparam(void) { return mlp_nparam(); }
int hss_predictor_nfeat(void) { return mlp_nfeat(); }

int hss_predictor_set(const float *W, const float *norm) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  try {
    if (!W || !norm) { c.pred_ready = false; return 0; }
    const int np = mlp_nparam(), nf = mlp_nfeat();
    std::vector<unsigned short> wb(np);
    for (int i = 0; i < np; ++i) {  // round to nearest even BF16
      unsigned int u;
      memcpy(&u, &W[i], 4);
      u += 0x7fff + ((u >> 16) & 1);
      wb[i] = (unsigned short)(u >> 16);
    }
    void *dw = buf<char>(c, "pred_wb", 2 * (size_t)np);
    float *dn = buf<float>(c, "pred_norm", 2 * (size_t)nf);
    CK(cudaMemcpy(dw, wb.data(), 2 * (size_t)np, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dn, norm, sizeof(float) * 2 * nf, cudaMemcpyHostToDevice));
    c.pred_ready = true;
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_predictor_features_dev(int k, const double *d, const double *z, double rho,
                               const double *difl, const double *difr, float *X, float *T,
                               void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (k < 0) return -1;
  if (k < 2) return 0;
  try {
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<int> s(1, 0), K(1, k), off{0, k};
    std::vector<double> r(1, rho);
    int *vs = buf<int>(c, "x_s", 1), *vK = buf<int>(c, "x_K", 1), *vo = buf<int>(c, "x_off", 2);
    double *vr = buf<double>(c, "x_rho", 1);
    h2d(vs, s, st); h2d(vK, K, st); h2d(vo, off, st); h2d(vr, r, st);
    LevelView lv{vs, vK, vr, vo, 1};
    float *feat = buf<float>(c, "x_feat", (size_t)k * (mlp_nfeat() + 1));
    launch_secular_mid(lv, k, k, d, z, feat, st);
    launch_train_targets(k, d, difl, difr, feat, X, T, st);
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_predictor_grad_dev(int n, const float *X, const float *T, const float *norm,
                           const float *W, float *G, float *loss, void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (n < 0) return -1;
  try {
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaMemsetAsync(G, 0, sizeof(float) * mlp_nparam(), st));
    CK(cudaMemsetAsync(loss, 0, sizeof(float), st));
    launch_mlp_grad(n, X, T, norm, W, G, loss, st);
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_predictor_adam_dev(const float *G, float *W, float *M, float *V, float lr, int step,
                           void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (step < 1) return -6;
  try {
    launch_adam(mlp_nparam(), W, G, M, V, lr, step, nullptr, (cudaStream_t)stream);
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

int hss_predict_dev(int k, const double *d, const double *z, double rho, float *guess,
                    void *stream) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (k < 0) return -1;
  if (!c.pred_ready) { c.err = "no predictor installed"; return 1; }
  try {
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<int> s(1, 0), K(1, k), off{0, k};
    std::vector<double> r(1, rho);
    int *vs = buf<int>(c, "x_s", 1), *vK = buf<int>(c, "x_K", 1), *vo = buf<int>(c, "x_off", 2);
    double *vr = buf<double>(c, "x_rho", 1);
    h2d(vs, s, st); h2d(vK, K, st); h2d(vo, off, st); h2d(vr, r, st);
    LevelView lv{vs, vK, vr, vo, 1};
    float *feat = buf<float>(c, "x_feat", (size_t)k * (mlp_nfeat() + 1));
    launch_secular_mid(lv, k, k, d, z, feat, st);
    launch_predict(k, feat, buf<char>(c, "pred_wb", 0), buf<float>(c, "pred_norm", 0), guess, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    return 0;
  } catch (CudaError &ex) {
    c.err = ex.msg;
    return 1000000;
  }
}

void cauchylike_(double *A, const double *D, const double *F, const double *u, const double *v,
                 const int *m_, const int *n_) {
  Ctx &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  const int m = *m_, n = *n_;
  if (m <= 0 || n <= 0) return;
  try {
    cudaStream_t st = nullptr;
    double *dD = buf<double>(c, "cl_D", m), *dF = buf<double>(c, "cl_F", n), *du = buf<double>(c, "cl_u", m),
           *dv = buf<double>(c, "cl_v", n), *dA = buf<double>(c, "cl_A", (size_t)m * n);
    CK(cudaMemcpyAsync(dD, D, sizeof(double) * m, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dF, F, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(du, u, sizeof(double) * m, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dv, v, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    launch_cauchylike(m, n, dD, dF, du, dv, dA, st);
    CK(cudaMemcpyAsync(A, dA, sizeof(double) * (size_t)m * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  } catch (CudaError &ex) {
    c.err = ex.msg;
  }
}

}  // extern "C"
