// Executors: the reference's wavelet entry points composed from the FP64
// kernels (ring DFTs, Wigner contractions, gamma DFTs, tiling merge), plus the
// C ABI wrappers (host-pointer drop-ins and device-pointer batch extensions).
//
// Data flow of one directional analysis at scale j (all maps of a batch at once):
//   flm --(l->t contraction, table D_n, weight conj psi_j(l,n))--> G_n[t][m]
//       --(gamma synthesis over n)--> spectra_g[t][m] --(inverse ring DFT)--> f_wav_j
// which fuses s2let_analysis_lm2lmn (src/c/s2let_analysis.c:28-89) with the SO3
// inverse (so3_core_inverse_direct, called at src/c/s2let_analysis.c:348): the
// normalisations 8pi^2/(2l+1), (2l+1)/(8pi^2), (-1)^n and sqrt((2l+1)/4pi)
// cancel, leaving conj(psi_j(l,n)) as the only per-l weight.  Synthesis runs the
// mirror image with the forward tables Q_n and merges all (j, n) in one kernel.
// The axisymmetric transforms are the same machinery with one direction (n = 0)
// per scale and the axisymmetric kernels as weights.
#include <algorithm>
#include <cstring>
#include <map>
#include <set>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "autotune.h"
#include "common.h"
#include "host_layer.h"
#include "kernels.h"
#include "mixed.h"
#include "plan.h"
#include "runtime.h"
#include "timing.h"

namespace s2g {

std::atomic<uint64_t> g_launches{0};
int current_kernel_type();  // host_layer.cpp
thread_local int t_precision = 0;
thread_local int t_table_mode = 0;  // 0 auto, 1 stored tables, 2 recomputed tables

namespace {

thread_local int t_status = 0;
thread_local std::string t_message;

int64_t table_budget_bytes();

template <class T>
T *upload(const std::vector<T> &v) {
  T *d = nullptr;
  S2G_CUDA(cudaMalloc(&d, sizeof(T) * std::max<size_t>(1, v.size())));
  if (!v.empty()) S2G_CUDA(cudaMemcpy(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return d;
}

// ---------------------------------------------------------------------------
// wavelet plan: one tiling (standard, manual or axisymmetric) of one signal type
// ---------------------------------------------------------------------------
struct Scale {
  int bl = 1, Nj = 1, ng = 1;
  int64_t woff = 0;              // offset of the scale in f_wav
  std::vector<int> ns;           // directions visited
  int *d_ns = nullptr;
  std::vector<int64_t> w_pair;   // per direction: [w(l,n) | w(l,-n)], 2*bl entries (merge weights)
  std::vector<int64_t> w_split;  // per direction: split weight, bl entries
  std::vector<int64_t> z_off;    // per direction: z block (bl^2) inside one map
  int64_t w_axi = -1;            // axisymmetric: per-l kernel weight (bl entries)
  // per direction: first l with a non-zero split / merge weight; terms below
  // are exact zeros and are skipped
  std::vector<int> lsup_split, lsup_merge;
};

struct WavPlan {
  int L = 0, s = 0;
  int ss = 0;  // sampling: 0 MW, 1 MWSS (rings and ring length per band-limit below)
  bool real = false, axisym = false;
  int bl_scal = 1, scal_lmin = 0;
  std::vector<Scale> sc;
  double2 *d_w = nullptr;
  int64_t w_phi = 0, w_cl = 0;
  MergePair *d_pairs = nullptr;
  int npairs = 0;
  int64_t z_per_map = 0;
  int max_bl = 1, max_nn = 1, max_ng = 1;
  std::vector<double2> w_host;  // host copy of d_w, for the kinds of its weight arrays
  // WKIND_* of the n weights at d_w + off
  int wkind(int64_t off, int n) const {
    bool re = true, im = true;
    for (int i = 0; i < n; ++i) {
      re = re && w_host[off + i].y == 0.0;
      im = im && w_host[off + i].x == 0.0;
    }
    return re ? WKIND_REAL : (im ? WKIND_IMAG : WKIND_COMPLEX);
  }
  std::vector<int> rc_bl;  // band-limits whose tables are recomputed (not stored)
  bool rc(int bl) const { return std::find(rc_bl.begin(), rc_bl.end(), bl) != rc_bl.end(); }
  const WignerTable &table(int bl, int an) const { return wigner_table(bl, an, ss, rc(bl)); }
  int nt(int bl) const { return grid_rings(bl, ss); }
  int K(int bl) const { return grid_ring_len(bl, ss); }
  void release() {
    cudaFree(d_w);
    cudaFree(d_pairs);
    for (auto &x : sc) cudaFree(x.d_ns);
    d_w = nullptr;
    d_pairs = nullptr;
  }
};

// Inputs of plan construction.
struct PlanSpec {
  int L = 0, spin = 0, ss = 0;
  bool real = false, axisym = false;
  int bl_scal = 1, scal_lmin = 0;
  std::vector<int> jrow, bl, Nj;  // per scale: psi row (or axisym kernel row), band-limits
  std::vector<int64_t> woff;      // per scale f_wav offsets
  const cplx *psi = nullptr;      // rows of L^2 (directional)
  const double *axi = nullptr;    // rows of L (axisymmetric kernels)
  const double *phi = nullptr;    // scaling weights, length L
  bool split_conj = true;         // split multiplies by conj(psi) (else psi)
  bool merge_conj = false;        // merge multiplies by conj(psi) (else psi)
};

std::unique_ptr<WavPlan> build_plan(const PlanSpec &ps) {
  auto P = std::make_unique<WavPlan>();
  P->L = ps.L;
  P->s = ps.real ? 0 : ps.spin;
  P->ss = ps.ss;
  P->real = ps.real;
  P->axisym = ps.axisym;
  P->bl_scal = ps.bl_scal;
  P->scal_lmin = ps.scal_lmin;
  const int L = ps.L;
  std::vector<double2> w;
  auto push = [&w](double re, double im) { w.push_back(make_double2(re, im)); };
  P->w_phi = 0;
  for (int l = 0; l < L; ++l) push(ps.phi[l], 0.0);
  P->w_cl = (int64_t)w.size();
  for (int l = 0; l < L; ++l) push(((P->s & 1) ? -1.0 : 1.0) * sqrt((2.0 * l + 1.0) / (4.0 * kPi)), 0.0);
  std::vector<MergePair> pairs;
  const int nsc = (int)ps.bl.size();
  P->sc.resize(nsc);
  for (int k = 0; k < nsc; ++k) {
    Scale &sd = P->sc[k];
    sd.bl = ps.bl[k];
    sd.Nj = ps.Nj[k];
    sd.woff = ps.woff[k];
    const int bl = sd.bl, jr = ps.jrow[k];
    if (ps.axisym) {
      sd.ns = {0};
      sd.ng = 1;
      sd.w_axi = (int64_t)w.size();
      for (int l = 0; l < bl; ++l) push(ps.axi[(size_t)jr * L + l], 0.0);
    } else {
      sd.ng = 2 * sd.Nj - 1;
      if (ps.real)
        for (int n = 1 - sd.Nj % 2; n < sd.Nj; n += 2) sd.ns.push_back(n);
      else
        for (int n = -sd.Nj + 1; n < sd.Nj; n += 2) sd.ns.push_back(n);
    }
    for (int n : sd.ns) {
      sd.w_pair.push_back((int64_t)w.size());
      for (int sgn = 0; sgn < 2; ++sgn) {
        const int nn = sgn == 0 ? n : -n;
        for (int l = 0; l < bl; ++l) {
          cplx v = 1.0;
          if (!ps.axisym) {
            v = (std::abs(nn) <= l) ? ps.psi[(size_t)jr * L * L + l * l + l + nn] : cplx(0.0);
            if (ps.merge_conj) v = std::conj(v);
          }
          push(v.real(), v.imag());
        }
      }
      sd.w_split.push_back((int64_t)w.size());
      for (int l = 0; l < bl; ++l) {
        cplx v = 1.0;
        if (!ps.axisym) {
          v = (std::abs(n) <= l) ? ps.psi[(size_t)jr * L * L + l * l + l + n] : cplx(0.0);
          if (ps.split_conj) v = std::conj(v);
        }
        push(v.real(), v.imag());
      }
      // weight supports: split = w_split, merge = w_pair halves (axisym: the kernel)
      auto first_nonzero = [&w, bl](int64_t off, int nrows) {
        for (int l = 0; l < bl; ++l)
          for (int r = 0; r < nrows; ++r) {
            const double2 v = w[off + (int64_t)r * bl + l];
            if (v.x != 0.0 || v.y != 0.0) return l;
          }
        return bl;
      };
      if (ps.axisym) {
        const int la = first_nonzero(sd.w_axi, 1);
        sd.lsup_split.push_back(la);
        sd.lsup_merge.push_back(la);
      } else {
        sd.lsup_split.push_back(first_nonzero(sd.w_split.back(), 1));
        sd.lsup_merge.push_back(first_nonzero(sd.w_pair.back(), 2));
      }
      sd.z_off.push_back(P->z_per_map);
      MergePair mp;
      mp.off = P->z_per_map;
      mp.bl = bl;
      mp.n = n;
      mp.lmin = std::max((ps.real || ps.axisym) ? 0 : std::abs(ps.spin), sd.lsup_merge.back());
      mp.woff = sd.w_pair.back();
      pairs.push_back(mp);
      P->z_per_map += (int64_t)bl * bl;
    }
    P->max_bl = std::max(P->max_bl, bl);
    P->max_nn = std::max(P->max_nn, (int)sd.ns.size());
    P->max_ng = std::max(P->max_ng, sd.ng);
  }
  P->npairs = (int)pairs.size();
  P->d_w = upload(w);
  P->w_host = w;
  P->d_pairs = upload(pairs);
  for (auto &sd : P->sc) sd.d_ns = upload(sd.ns);
  // stored or recomputed tables: stored while the plan's tables fit the budget,
  // else the largest band-limits are recomputed first
  {
    std::map<int, std::set<int>> need;  // bl -> |n|
    need[L].insert(std::abs(P->s));
    need[ps.bl_scal].insert(0);
    for (auto &sd : P->sc)
      for (int n : sd.ns) need[sd.bl].insert(std::abs(n));
    std::map<int, int64_t> bytes;
    int64_t total = 0;
    for (auto &kv : need)
      for (int an : kv.second) {
        const int64_t b = stored_table_bytes(kv.first, an, P->ss);
        bytes[kv.first] += b;
        total += b;
      }
    if (t_table_mode == 2) {
      for (auto &kv : need) P->rc_bl.push_back(kv.first);
    } else if (t_table_mode == 0) {
      const int64_t budget = table_budget_bytes();
      for (auto it = need.rbegin(); it != need.rend() && total > budget; ++it) {
        P->rc_bl.push_back(it->first);
        total -= bytes[it->first];
      }
    }
  }
  // build the Wigner tables and FFT data now, outside the transforms' timing
  P->table(L, std::abs(P->s));
  P->table(ps.bl_scal, 0);
  for (auto &sd : P->sc)
    for (int n : sd.ns) P->table(sd.bl, std::abs(n));
  ring_fft(P->K(L));
  ring_fft(P->K(ps.bl_scal));
  for (auto &sd : P->sc) ring_fft(P->K(sd.bl));
  return P;
}

// standard (tiling from the parameters), cached per parameter set ------------
struct PlanKey {
  int L, J_min, N, spin, original_spin, upsample, reality, real, axisym, multires, kernel, sampling, table_mode;
  double B;
  bool operator<(const PlanKey &o) const { return std::memcmp(this, &o, sizeof(PlanKey)) < 0; }
};
std::mutex g_plan_mu;
std::map<PlanKey, std::unique_ptr<WavPlan>> g_plans;

const WavPlan &directional_plan(const s2let_parameters_t &p, bool real) {
  PlanKey key;
  std::memset(&key, 0, sizeof key);
  key.L = p.L;
  key.J_min = p.J_min;
  key.N = p.N;
  key.spin = real ? 0 : p.spin;
  key.original_spin = p.original_spin;
  key.upsample = p.upsample;
  key.reality = p.reality;
  key.real = real;
  key.kernel = current_kernel_type();
  key.sampling = p.sampling_scheme;
  key.table_mode = t_table_mode;
  key.B = p.B;
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto it = g_plans.find(key);
  if (it != g_plans.end()) return *it->second;
  s2let_parameters_t q = p;
  if (real) {
    q.reality = 1;
    q.spin = 0;
  }
  const Layout g = make_layout(q, real);
  const int L = p.L;
  std::vector<cplx> psi((size_t)(g.J + 1) * L * L, 0.0);
  std::vector<double> phi(L, 0.0);
  tiling_wavelet(psi.data(), phi.data(), q);
  PlanSpec ps;
  ps.L = L;
  ps.spin = q.spin;
  ps.ss = p.sampling_scheme == S2LET_SAMPLING_MW_SS ? 1 : 0;
  ps.real = real;
  ps.bl_scal = g.bl_scal;
  ps.jrow = g.j;
  ps.bl = g.bl;
  ps.Nj = g.Nj;
  ps.woff.assign(g.woff.begin(), g.woff.end() - 1);
  ps.psi = psi.data();
  ps.phi = phi.data();
  auto P = build_plan(ps);
  const WavPlan &ref = *P;
  g_plans.emplace(key, std::move(P));
  return ref;
}

const WavPlan &axisym_plan(const s2let_parameters_t &p, bool real, bool multires) {
  PlanKey key;
  std::memset(&key, 0, sizeof key);
  key.L = p.L;
  key.J_min = p.J_min;
  key.real = real;
  key.axisym = 1;
  key.multires = multires;
  key.kernel = current_kernel_type();
  key.table_mode = t_table_mode;
  key.B = p.B;
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto it = g_plans.find(key);
  if (it != g_plans.end()) return *it->second;
  const int L = p.L, J = j_max(p);
  std::vector<double> wav((size_t)(J + 1) * L, 0.0), scal(L, 0.0);
  axisym_kernels(wav.data(), scal.data(), p);
  PlanSpec ps;
  ps.L = L;
  ps.spin = 0;
  ps.real = real;
  ps.axisym = true;
  ps.bl_scal = multires ? std::min(bandlimit(p.J_min - 1, p), L) : L;
  int64_t off = 0;
  for (int j = p.J_min; j <= J; ++j) {
    const int bl = multires ? std::min(bandlimit(j, p), L) : L;
    ps.jrow.push_back(j);
    ps.bl.push_back(bl);
    ps.Nj.push_back(1);
    ps.woff.push_back(off);
    off += (int64_t)bl * (2 * bl - 1);
  }
  ps.axi = wav.data();
  ps.phi = scal.data();
  auto P = build_plan(ps);
  const WavPlan &ref = *P;
  g_plans.emplace(key, std::move(P));
  return ref;
}

// ---------------------------------------------------------------------------
// full-band spin-s spherical-harmonic transforms (MW or MWSS)
// ---------------------------------------------------------------------------

struct Sht {
  int L, s, ss;
  bool real;
  const double2 *cl;  // (-1)^s sqrt((2l+1)/4pi), l < L (device)
  bool rc;            // recomputed table
};
Sht sht_of(const WavPlan &P) { return Sht{P.L, P.s, P.ss, P.real, P.d_w + P.w_cl, P.rc(P.L)}; }

// flm (nb x L^2, zero outside the computed range) <- forward transform of maps
// (or the adjoint of the inverse)
void sht_forward_once(const Sht &H, const void *f, int64_t fstride, double2 *flm, int nb, Scratch &S,
                      bool adjoint_of_inverse) {
  const int L = H.L, s = H.s, K = grid_ring_len(L, H.ss), nt = grid_rings(L, H.ss);
  const bool real = H.real;
  const int sw = real ? L : 2 * L - 1, mlo = real ? 0 : -(L - 1);
  double2 *spec = S.get<double2>((int64_t)nb * nt * sw);
  ring_forward(f, K, fstride, nt, spec, sw, sw, mlo, nb * nt, L, H.ss, real, S.st);
  S2G_CUDA(cudaMemsetAsync(flm, 0, sizeof(double2) * nb * L * L, S.st));
  T2L a{};
  a.tb = &wigner_table(L, std::abs(s), H.ss, H.rc);
  a.n = -s;
  a.use_q = !adjoint_of_inverse;
  a.mlo = mlo;
  a.mhi = L - 1;
  a.in = spec;
  a.is = (int64_t)nt * sw;
  a.iw = sw;
  a.imlo = mlo;
  a.w = H.cl;
  a.wkind = WKIND_REAL;
  a.wscale = adjoint_of_inverse ? 1.0 : 2.0 * kPi / K;
  a.lmin = std::abs(s);
  a.y = flm;
  a.ys = (int64_t)L * L;
  a.nb = nb;
  contract_t2l(a, S.st);
}

// maps <- inverse transform (or adjoint of the forward) of flm
void sht_inverse(const Sht &H, const double2 *flm, bool flm_half, void *f, int64_t fstride, int nb,
                 Scratch &S, bool adjoint_of_forward) {
  const int L = H.L, s = H.s, K = grid_ring_len(L, H.ss), nt = grid_rings(L, H.ss);
  const bool real = H.real;
  const int sw = real ? L : 2 * L - 1, mlo = real ? 0 : -(L - 1);
  double2 *spec = S.get<double2>((int64_t)nb * nt * sw);
  L2T a{};
  a.tb = &wigner_table(L, std::abs(s), H.ss, H.rc);
  a.n = -s;
  a.use_q = adjoint_of_forward;
  a.mlo = mlo;
  a.mhi = L - 1;
  a.x = flm;
  a.xs = (int64_t)L * L;
  a.xL = L;
  a.x_half = flm_half;
  a.w = H.cl;
  a.wkind = WKIND_REAL;
  a.wscale = adjoint_of_forward ? 2.0 * kPi / K : 1.0;
  a.lmin = std::abs(s);
  a.out = spec;
  a.os = (int64_t)nt * sw;
  a.ow = sw;
  a.omlo = mlo;
  a.nb = nb;
  contract_l2t(a, S.st);
  ring_inverse(spec, sw, sw, mlo, f, K, fstride, nt, nb * nt, L, H.ss, real, S.st);
}

// Forward transform with one residual-refinement sweep (FP64 path, L above
// kRefineL): flm += F(f - I(flm)).  The direct-theta quadrature projects the
// high degrees out of ring spectra dominated by the low ones, so its FP64
// rounding grows like l^2 eps relative to those coefficients for steep spectra
// (measured per degree against a quad-precision map: 5e-14 at L = 512, ~1e-12
// at L = 2048).  For band-limited maps the residual is at rounding level and
// the sweep brings the coefficients back to the FFT-based quadrature's
// accuracy; for other maps F(f - I(F f)) vanishes in exact arithmetic and the
// sweep changes nothing beyond rounding.
constexpr int kRefineL = 1024;

void sht_forward(const Sht &H, const void *f, int64_t fstride, double2 *flm, int nb, Scratch &S,
                 bool adjoint_of_inverse) {
  sht_forward_once(H, f, fstride, flm, nb, S, adjoint_of_inverse);
  if (adjoint_of_inverse || t_precision != 0 || H.L <= kRefineL || nb <= 0) return;
  const int64_t npx = (int64_t)grid_rings(H.L, H.ss) * grid_ring_len(H.L, H.ss);
  const int64_t dd = H.real ? 1 : 2;  // doubles per sample
  const int64_t L2 = (int64_t)H.L * H.L;
  double *r = S.get<double>(nb * npx * dd);
  double2 *dflm = S.get<double2>(nb * L2);
  sht_inverse(H, flm, H.real, r, npx, nb, S, false);                           // r = I(flm)
  axpby((const double *)f, fstride * dd, r, npx * dd, npx * dd, nb, 1.0, -1.0, S.st);  // r = f - r
  sht_forward_once(H, r, npx, dflm, nb, S, false);
  axpby((const double *)dflm, 2 * L2, (double *)flm, 2 * L2, 2 * L2, nb, 1.0, 1.0, S.st);  // flm += dflm
}

// ---------------------------------------------------------------------------
// harmonic <-> wavelet space
// ---------------------------------------------------------------------------

enum SplitMode { SPLIT_ANALYSIS, SPLIT_SYNTH_ADJ };
enum MergeMode { MERGE_SYNTHESIS, MERGE_ANALYSIS_ADJ };

// Host f_wav copies overlapped with the transforms of one batch.  A piece is
// one scale of a group of consecutive maps: elements woff .. woff + len of
// each map's f_wav (seglen[woff] = len).  Analysis: the copy stream takes each
// piece to the host as soon as the kernels on the compute stream have written
// it.  Synthesis: every piece is queued on the copy stream up front, in the
// order the transforms read them, and the compute stream waits for a piece's
// event before its first kernel reads it.
struct WavPipe {
  cudaStream_t cs = nullptr;  // copy stream
  char *host = nullptr;       // map b's f_wav at host + b * hstride * esz
  int64_t hstride = 0;
  size_t esz = 0;
  int group = 8;                           // maps per piece
  std::map<int64_t, int64_t> seglen;       // scale offset -> elements of the scale
  std::map<std::pair<int64_t, int>, cudaEvent_t> ready;  // (scale offset, first map) -> copied in
  std::vector<cudaEvent_t> events;
  WavPipe() = default;
  WavPipe(const WavPipe &) = delete;
  WavPipe &operator=(const WavPipe &) = delete;
  ~WavPipe() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  }
  cudaEvent_t event() {
    cudaEvent_t e;
    S2G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    events.push_back(e);
    return e;
  }
  // analysis: piece (woff, maps b0 .. b0 + nbg) written by the kernels queued so far on st
  void out(cudaStream_t st, const void *dev, int64_t dstride, int64_t woff, int b0, int nbg) {
    cudaEvent_t e = event();
    S2G_CUDA(cudaEventRecord(e, st));
    S2G_CUDA(cudaStreamWaitEvent(cs, e, 0));
    const int64_t len = seglen.at(woff);
    copy_async(host + ((size_t)b0 * hstride + woff) * esz, hstride * esz,
               (const char *)dev + ((size_t)b0 * dstride + woff) * esz, dstride * esz, len * esz, nbg,
               cudaMemcpyDeviceToHost, cs);
  }
  // synthesis: queue the copy of piece (woff, b0 .. b0 + nbg) into dev
  void in(void *dev, int64_t dstride, int64_t woff, int b0, int nbg) {
    const int64_t len = seglen.at(woff);
    copy_async((char *)dev + ((size_t)b0 * dstride + woff) * esz, dstride * esz,
               host + ((size_t)b0 * hstride + woff) * esz, hstride * esz, len * esz, nbg, cudaMemcpyHostToDevice,
               cs);
    cudaEvent_t e = event();
    S2G_CUDA(cudaEventRecord(e, cs));
    ready[{woff, b0}] = e;
  }
  // synthesis: the compute stream waits for piece (woff, b0)
  void wait(cudaStream_t st, int64_t woff, int b0) {
    auto it = ready.find({woff, b0});
    S2G_REQUIRE(it != ready.end(), ERR_INVALID, "host pipeline: piece not queued");
    S2G_CUDA(cudaStreamWaitEvent(st, it->second, 0));
  }
};
const double kSqrt2Pi = 2.5066282746310005024;

// flm -> (f_wav, f_scal).  SPLIT_ANALYSIS: lm2wav.  SPLIT_SYNTH_ADJ: adjoint of wav2lm.
// Ring DFTs per theta ring on the nn n-components (one complex DFT each) when
// that is fewer than on the ng gamma slices (real slices pair up, two per
// complex DFT); the gamma DFT then runs on pixels.
bool rings_on_n(const WavPlan &P, const Scale &sd) {
  const double on_n = (double)sd.ns.size();
  const double on_g = P.real ? 0.5 * sd.ng : (double)sd.ng;
  return on_n < on_g;
}

// Whether some scale of the plan runs its ring and gamma DFTs as separate
// launches through a ring buffer (the fused launch keeps them on chip).
bool needs_ring_buffer(const WavPlan &P) {
  for (const Scale &sd : P.sc)
    if (!rings_on_n(P, sd) || !ring_gamma_fusable((int)sd.ns.size(), sd.ng, sd.bl, P.ss)) return true;
  return false;
}

// Scale ranges [k0, k1) that share one table pass (consecutive scales with the
// same band-limit and directions), smallest band-limits first, or largest
// first when `largest_first`.
std::vector<std::pair<size_t, size_t>> table_passes(const WavPlan &P, bool largest_first) {
  std::vector<std::pair<size_t, size_t>> passes;
  for (size_t k0 = 0; k0 < P.sc.size();) {
    size_t k1 = k0 + 1;
    if (k1 < P.sc.size() && P.sc[k1].bl == P.sc[k0].bl && P.sc[k1].ns == P.sc[k0].ns) ++k1;
    passes.emplace_back(k0, k1);
    k0 = k1;
  }
  if (largest_first) std::reverse(passes.begin(), passes.end());
  return passes;
}

void wav_split(const WavPlan &P, SplitMode mode, const double2 *flm, bool flm_half, void *f_wav,
               int64_t wstride, void *f_scal, int64_t sstride, int nb, Scratch &S, WavPipe *pipe = nullptr) {
  const bool real = P.real;
  const int L = P.L;
  const size_t esz = real ? sizeof(double) : sizeof(double2);
  const bool adj = (mode == SPLIT_SYNTH_ADJ);
  // scaling function: spin-0 transform at bl_scal
  {
    const int bs = P.bl_scal, Ks = P.K(bs), nts = P.nt(bs);
    const int sw = real ? bs : 2 * bs - 1, mlo = real ? 0 : -(bs - 1);
    double2 *spec = S.get<double2>((int64_t)nb * nts * sw);
    L2T a{};
    a.tb = &P.table(bs, 0);
    a.n = 0;
    a.use_q = adj;
    a.mlo = mlo;
    a.mhi = bs - 1;
    a.x = flm;
    a.xs = (int64_t)L * L;
    a.xL = L;
    a.x_half = flm_half;
    a.w = P.d_w + P.w_phi;
    a.wkind = P.wkind(P.w_phi, bs);
    a.wscale = adj ? 2.0 * kPi / Ks : 1.0;
    a.lmin = P.scal_lmin;
    a.out = spec;
    a.os = (int64_t)nts * sw;
    a.ow = sw;
    a.omlo = mlo;
    a.nb = nb;
    contract_l2t(a, S.st);
    ring_inverse(spec, sw, sw, mlo, f_scal, Ks, sstride, nts, nb * nts, bs, P.ss, real, S.st);
  }
  // G buffers [b][n][t][m] (spectral width W = 2bl-1), ring buffers [b][n or g][t][p]
  const int64_t Wmax = 2 * P.max_bl - 1, Kmax = 2 * P.max_bl, ntmax = P.nt(P.max_bl);
  const int64_t gsz = (int64_t)nb * P.max_nn * ntmax * Wmax;
  double2 *Gbuf = S.get<double2>(2 * gsz);
  // ring buffers only for the scales whose ring and gamma DFTs are separate launches
  double2 *spec = needs_ring_buffer(P) ? S.get<double2>((int64_t)nb * std::max(P.max_ng, P.max_nn) * ntmax * Kmax)
                                       : nullptr;
  // with host copies the largest scales go first, so that most of f_wav can
  // cross the bus while the smaller scales are transformed
  const std::vector<std::pair<size_t, size_t>> passes = table_passes(P, pipe != nullptr);
  for (const auto &pk : passes) {
    const size_t k0 = pk.first, k1 = pk.second;
    const int ngrp = (int)(k1 - k0);
    const int bl = P.sc[k0].bl, W = 2 * bl - 1, nn = (int)P.sc[k0].ns.size();
    const int nt = P.nt(bl), K = P.K(bl);
    for (int i = 0; i < nn; ++i) {
      L2T grp[2];
      for (int q = 0; q < ngrp; ++q) {
        const Scale &sd = P.sc[k0 + q];
        const int n = sd.ns[i];
        L2T &a = grp[q];
        a = L2T{};
        a.tb = &P.table(bl, std::abs(n));
        a.n = n;
        a.use_q = adj;
        a.mlo = (real && n == 0) ? 0 : -(bl - 1);
        a.mhi = bl - 1;
        a.x = flm;
        a.xs = (int64_t)L * L;
        a.xL = L;
        a.x_half = flm_half;
        if (P.axisym) {
          a.w = P.d_w + sd.w_axi;
          a.wkind = P.wkind(sd.w_axi, bl);
          a.wscale = adj ? 2.0 * kPi / K * kSqrt2Pi : 1.0 / kSqrt2Pi;
        } else {
          a.w = P.d_w + sd.w_split[i];
          a.wkind = P.wkind(sd.w_split[i], bl);
          a.wscale = adj ? 4.0 * kPi * kPi / K : 1.0;
        }
        a.lmin = std::max((real || P.axisym) ? 0 : std::abs(P.s), sd.lsup_split[i]);
        a.out = Gbuf + q * gsz + (int64_t)i * nt * W;
        a.os = (int64_t)nn * nt * W;
        a.ow = W;
        a.omlo = -(bl - 1);
        a.nb = nb;
      }
      contract_l2t_group(grp, ngrp, S.st);
    }
    for (int q = 0; q < ngrp; ++q) {
      const Scale &sd = P.sc[k0 + q];
      const int ng = sd.ng;
      const double c = adj && !P.axisym ? 1.0 / ng : 1.0;
      char *out = (char *)f_wav + (size_t)sd.woff * esz;
      const double2 *Gq = Gbuf + q * gsz;
      if (rings_on_n(P, sd)) {
        // F_n(t, p) = sum_m G_n(t, m) e^{i m phi_p}; spec holds F[b][i][t][p].
        // With host copies, in groups of maps, each group copied out when done.
        const int G = pipe ? pipe->group : nb;
        for (int b0 = 0; b0 < nb; b0 += G) {
          const int nbg = std::min(G, nb - b0);
          const double2 *Gb = Gq + (int64_t)b0 * nn * nt * W;
          if (ring_gamma_fusable(nn, ng, bl, P.ss)) {  // one launch, the n-components stay on chip
            ring_inverse_gamma(Gb, (int64_t)nn * nt * W, (int64_t)nt * W, sd.ns, ng, real, c,
                               out + (size_t)b0 * wstride * esz, wstride, nbg, bl, P.ss, S.st);
            if (pipe) pipe->out(S.st, f_wav, wstride, sd.woff, b0, nbg);
            continue;
          }
          double2 *sb = spec + (int64_t)b0 * nn * nt * K;
          for (int i = 0; i < nn; ++i) {
            const bool herm = real && sd.ns[i] == 0;  // real signal, n = 0: only m >= 0 computed
            ring_inverse_c(Gb + (int64_t)i * nt * W + (herm ? bl - 1 : 0), W, (int64_t)nn * nt * W, nt,
                           herm ? bl : W, herm ? 0 : -(bl - 1), herm, sb + (int64_t)i * nt * K, K,
                           (int64_t)nn * nt * K, nt, nbg * nt, bl, P.ss, S.st);
          }
          gamma_px_synthesis(sb, out + (size_t)b0 * wstride * esz, wstride, sd.d_ns, nn, ng, bl, P.ss, nbg, real,
                             c, S.st);
          if (pipe) pipe->out(S.st, f_wav, wstride, sd.woff, b0, nbg);
        }
      } else {
        const int sw = real ? bl : W, mlo = real ? 0 : -(bl - 1);
        gamma_synthesis(Gq, spec, sd.d_ns, nn, ng, bl, P.ss, nb, real, c, S.st);
        ring_inverse(spec, sw, sw, mlo, out, K, wstride, ng * nt, nb * ng * nt, bl, P.ss, real, S.st);
        if (pipe) pipe->out(S.st, f_wav, wstride, sd.woff, 0, nb);
      }
    }
  }
}

// (f_wav, f_scal) -> flm.  MERGE_SYNTHESIS: wav2lm.  MERGE_ANALYSIS_ADJ: adjoint of lm2wav.
// For real signals flm holds m >= 0 only.  accumulate: add to flm instead of overwriting.
void wav_merge(const WavPlan &P, MergeMode mode, const void *f_wav, int64_t wstride, const void *f_scal,
               int64_t sstride, double2 *flm, int nb, Scratch &S, bool accumulate = false,
               WavPipe *pipe = nullptr) {
  const bool real = P.real;
  const int L = P.L;
  const size_t esz = real ? sizeof(double) : sizeof(double2);
  const bool adj = (mode == MERGE_ANALYSIS_ADJ);
  double2 *z = S.get<double2>((int64_t)nb * std::max<int64_t>(1, P.z_per_map));
  const int bs = P.bl_scal, Ks = P.K(bs), nts = P.nt(bs);
  double2 *zs = S.get<double2>((int64_t)nb * bs * bs);
  {
    const int sw = real ? bs : 2 * bs - 1, mlo = real ? 0 : -(bs - 1);
    double2 *spec = S.get<double2>((int64_t)nb * nts * sw);
    ring_forward(f_scal, Ks, sstride, nts, spec, sw, sw, mlo, nb * nts, bs, P.ss, real, S.st);
    if (P.scal_lmin > 0) S2G_CUDA(cudaMemsetAsync(zs, 0, sizeof(double2) * nb * bs * bs, S.st));
    T2L a{};
    a.tb = &P.table(bs, 0);
    a.n = 0;
    a.use_q = !adj;
    a.mlo = mlo;
    a.mhi = bs - 1;
    a.in = spec;
    a.is = (int64_t)nts * sw;
    a.iw = sw;
    a.imlo = mlo;
    a.w = P.d_w + P.w_phi;
    a.wkind = P.wkind(P.w_phi, bs);
    a.wscale = adj ? 1.0 : 2.0 * kPi / Ks;
    a.lmin = P.scal_lmin;
    a.y = zs;
    a.ys = (int64_t)bs * bs;
    a.nb = nb;
    contract_t2l(a, S.st);
  }
  const int64_t Wmax = 2 * P.max_bl - 1, Kmax = 2 * P.max_bl, ntmax = P.nt(P.max_bl);
  const int64_t gsz = (int64_t)nb * P.max_nn * ntmax * Wmax;
  double2 *Gbuf = S.get<double2>(2 * gsz);
  double2 *spec = needs_ring_buffer(P) ? S.get<double2>((int64_t)nb * std::max(P.max_ng, P.max_nn) * ntmax * Kmax)
                                       : nullptr;
  // with host copies the largest scales go first (their pieces are queued
  // first, see merge_order), so that their ring DFTs run while the rest of
  // f_wav is still crossing the bus
  const std::vector<std::pair<size_t, size_t>> passes = table_passes(P, pipe != nullptr);
  for (const auto &pk : passes) {
    const size_t k0 = pk.first, k1 = pk.second;
    const int ngrp = (int)(k1 - k0);
    const int bl = P.sc[k0].bl, W = 2 * bl - 1, nn = (int)P.sc[k0].ns.size();
    const int nt = P.nt(bl), K = P.K(bl);
    const int sw = real ? bl : W, mlo = real ? 0 : -(bl - 1);
    for (int q = 0; q < ngrp; ++q) {
      const Scale &sd = P.sc[k0 + q];
      const int ng = sd.ng;
      const double c = (adj || P.axisym) ? 1.0 : 1.0 / ng;
      const char *in = (const char *)f_wav + (size_t)sd.woff * esz;
      double2 *Gq = Gbuf + q * gsz;
      if (rings_on_n(P, sd)) {
        // F_n(t, p) = c sum_g e^{-i n gamma_g} f_g(t, p), then one DFT per (n, t).
        // With host copies, in groups of maps, each after its copy has landed.
        const int G = pipe ? pipe->group : nb;
        for (int b0 = 0; b0 < nb; b0 += G) {
          const int nbg = std::min(G, nb - b0);
          if (pipe) pipe->wait(S.st, sd.woff, b0);
          if (ring_gamma_fusable(nn, ng, bl, P.ss)) {  // one launch, the n-components stay on chip
            gamma_ring_forward(in + (size_t)b0 * wstride * esz, wstride, sd.ns, ng, real, c,
                               Gq + (int64_t)b0 * nn * nt * W, (int64_t)nn * nt * W, (int64_t)nt * W, nbg, bl, P.ss,
                               S.st);
            continue;
          }
          double2 *sb = spec + (int64_t)b0 * nn * nt * K;
          gamma_px_analysis(in + (size_t)b0 * wstride * esz, wstride, sb, sd.d_ns, nn, ng, bl, P.ss, nbg, real, c,
                            S.st);
          for (int i = 0; i < nn; ++i)
            ring_forward_c(sb + (int64_t)i * nt * K, K, (int64_t)nn * nt * K, nt,
                           Gq + (int64_t)b0 * nn * nt * W + (int64_t)i * nt * W, W, (int64_t)nn * nt * W, nt, W,
                           -(bl - 1), nbg * nt, bl, P.ss, S.st);
        }
      } else {
        if (pipe) pipe->wait(S.st, sd.woff, 0);
        ring_forward(in, K, wstride, ng * nt, spec, sw, sw, mlo, nb * ng * nt, bl, P.ss, real, S.st);
        gamma_analysis(spec, Gq, sd.d_ns, nn, ng, bl, P.ss, nb, real, c, S.st);
      }
    }
    for (int i = 0; i < nn; ++i) {
      T2L grp[2];
      for (int q = 0; q < ngrp; ++q) {
        const Scale &sd = P.sc[k0 + q];
        const int n = sd.ns[i];
        T2L &a = grp[q];
        a = T2L{};
        a.tb = &P.table(bl, std::abs(n));
        a.n = n;
        a.use_q = !adj;
        a.mlo = (real && n == 0) ? 0 : -(bl - 1);
        a.mhi = bl - 1;
        a.in = Gbuf + q * gsz + (int64_t)i * nt * W;
        a.is = (int64_t)nn * nt * W;
        a.iw = W;
        a.imlo = -(bl - 1);
        if (P.axisym) {
          a.w = P.d_w + sd.w_axi;
          a.wkind = P.wkind(sd.w_axi, bl);
          a.wscale = adj ? 1.0 / kSqrt2Pi : 2.0 * kPi / K * kSqrt2Pi;
          a.lmin = sd.lsup_merge[i];
        } else {
          a.w = nullptr;
          a.wscale = adj ? 1.0 : 4.0 * kPi * kPi / K;
          a.lmin = std::max(real ? 0 : std::abs(P.s), sd.lsup_merge[i]);
        }
        a.y = z + sd.z_off[i];
        a.ys = P.z_per_map;
        a.nb = nb;
      }
      contract_t2l_group(grp, ngrp, S.st);
    }
  }
  merge_lmn(flm, L, (int64_t)L * L, z, P.z_per_map, P.d_pairs, P.npairs, P.d_w, zs, (int64_t)bs * bs, bs,
            real, accumulate, nb, S.st);
}

// Device bytes that stored tables of one plan may take: 60 % of the memory
// free when the plan is built (S2LET_GPU_TABLE_BUDGET_GB overrides).
int64_t table_budget_bytes() {
  const char *e = getenv("S2LET_GPU_TABLE_BUDGET_GB");
  if (e && e[0]) return (int64_t)(atof(e) * 1073741824.0);
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return INT64_MAX;
  return (int64_t)(0.6 * (double)fr);
}

// (-1)^s sqrt((2l+1)/4pi) on the device, cached per (L, s)
const double2 *cl_weights(int L, int s) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, double2 *> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(L, s);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  std::vector<double2> w(L);
  for (int l = 0; l < L; ++l) w[l] = make_double2(((s & 1) ? -1.0 : 1.0) * sqrt((2.0 * l + 1.0) / (4.0 * kPi)), 0.0);
  double2 *d = upload(w);
  cache[key] = d;
  return d;
}

}  // namespace

// ---------------------------------------------------------------------------
// status / runtime helpers (declared in runtime.h)
// ---------------------------------------------------------------------------

void set_status(int code, const std::string &msg) {
  t_status = code;
  t_message = msg;
}
void report_failure() {
  fprintf(stderr, "s2let_gpu: %s\n", t_message.c_str());
  const char *ab = getenv("S2LET_GPU_ABORT_ON_ERROR");
  if (ab && ab[0] == '1') exit(1);
}
int last_status() { return t_status; }

// The device this process's library works on: the one current at the first
// compute call (or named by s2let_gpu_bind_device).  Plans, Wigner tables,
// streams and kernel attributes are cached process-wide for that device only,
// so a call made while another device is current is refused.
std::atomic<int> g_bound_device{-1};

int bind_device(int dev) {
  if (dev < 0) return ERR_INVALID;
  int expected = -1;
  if (g_bound_device.compare_exchange_strong(expected, dev) || expected == dev) return OK;
  return ERR_UNSUPPORTED;
}

void ensure_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  S2G_REQUIRE(e == cudaSuccess && n > 0, ERR_NO_DEVICE, "no CUDA device available");
  int dev = -1;
  S2G_CUDA(cudaGetDevice(&dev));
  if (bind_device(dev) != OK)
    throw Error(ERR_UNSUPPORTED, "the library serves CUDA device " + std::to_string(g_bound_device.load()) +
                                     " in this process (its first device); device " + std::to_string(dev) +
                                     " is current: make device " + std::to_string(g_bound_device.load()) +
                                     " current, or use one process per device");
  static std::once_flag f;
  std::call_once(f, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;  // keep freed scratch cached in the pool
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  });
}

cudaStream_t host_stream() {
  static thread_local cudaStream_t st = nullptr;
  if (!st) S2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  return st;
}

namespace {
}  // namespace

// ===========================================================================
// executors (device pointers, one stream)
// ===========================================================================

enum Op { OP_PX2WAV, OP_WAV2PX, OP_ADJ_WAV2PX, OP_ADJ_PX2WAV, OP_LM2WAV, OP_WAV2LM, OP_ADJ_WAV2LM,
          OP_ADJ_LM2WAV };

// One wavelet transform of `nb` maps with plan P.  Pixel maps, wavelet and
// scaling arrays are batched with their single-map sizes as strides.
void run_plan(Op op, const WavPlan &P, void *px, void *lm, void *wav, int64_t nw, void *scal, int64_t ns,
              int nb, cudaStream_t st, bool accumulate_lm = false, WavPipe *pipe = nullptr) {
  if (nb <= 0) return;
  Scratch S(st);
  const int L = P.L;
  const bool real = P.real;
  const int64_t npx = (int64_t)P.nt(L) * P.K(L);
  const bool lm_api = (op == OP_LM2WAV || op == OP_WAV2LM || op == OP_ADJ_WAV2LM || op == OP_ADJ_LM2WAV);
  double2 *flm = lm_api ? (double2 *)lm : S.get<double2>((int64_t)nb * L * L);
  switch (op) {
  case OP_PX2WAV:
    sht_forward(sht_of(P), px, npx, flm, nb, S, false);
    wav_split(P, SPLIT_ANALYSIS, flm, real, wav, nw, scal, ns, nb, S, pipe);
    break;
  case OP_LM2WAV:
    wav_split(P, SPLIT_ANALYSIS, flm, false, wav, nw, scal, ns, nb, S);
    break;
  case OP_ADJ_PX2WAV:
    sht_forward(sht_of(P), px, npx, flm, nb, S, true);
    wav_split(P, SPLIT_SYNTH_ADJ, flm, real, wav, nw, scal, ns, nb, S, pipe);
    break;
  case OP_ADJ_LM2WAV:
    wav_split(P, SPLIT_SYNTH_ADJ, flm, false, wav, nw, scal, ns, nb, S);
    break;
  case OP_WAV2PX:
    wav_merge(P, MERGE_SYNTHESIS, wav, nw, scal, ns, flm, nb, S, false, pipe);
    sht_inverse(sht_of(P), flm, real, px, npx, nb, S, false);
    break;
  case OP_WAV2LM:
    wav_merge(P, MERGE_SYNTHESIS, wav, nw, scal, ns, flm, nb, S, accumulate_lm);
    if (real) symmetrize_flm(flm, L, (int64_t)L * L, nb, st);
    break;
  case OP_ADJ_WAV2PX:
    wav_merge(P, MERGE_ANALYSIS_ADJ, wav, nw, scal, ns, flm, nb, S, false, pipe);
    sht_inverse(sht_of(P), flm, real, px, npx, nb, S, true);
    break;
  case OP_ADJ_WAV2LM:
    wav_merge(P, MERGE_ANALYSIS_ADJ, wav, nw, scal, ns, flm, nb, S, accumulate_lm);
    if (real) symmetrize_flm(flm, L, (int64_t)L * L, nb, st);
    break;
  }
}

void run_directional(Op op, const s2let_parameters_t &p, bool real, void *px, void *lm, void *wav,
                     void *scal, int nb, cudaStream_t st) {
  validate(&p);
  const WavPlan &P = directional_plan(p, real);
  run_plan(op, P, px, lm, wav, s2let_n_wav(&p), scal, s2let_n_scal(&p), nb, st);
}

// Plain spherical-harmonic transform on device buffers, MW (ss = 0) or MWSS
// (ss = 1) sampling.  dir: 0 forward (map -> flm), 1 inverse, 2 adjoint of
// forward (flm -> map), 3 adjoint of inverse (map -> flm).  Real signals: flm
// returned complete.
void run_sht(int dir, int L, int spin, bool real, int ss, void *f, double2 *flm, int nb, cudaStream_t st) {
  S2G_REQUIRE(L >= 1 && L <= 8192, ERR_INVALID, "L must lie in [1, 8192]");
  S2G_REQUIRE(std::abs(spin) < L, ERR_INVALID, "|spin| must be < L");
  if (real) S2G_REQUIRE(spin == 0, ERR_INVALID, "real signals are spin 0");
  Scratch S(st);
  bool rc = t_table_mode == 2;
  if (t_table_mode == 0) rc = stored_table_bytes(L, std::abs(real ? 0 : spin), ss) > table_budget_bytes();
  const Sht H{L, real ? 0 : spin, ss, real, cl_weights(L, real ? 0 : spin), rc};
  wigner_table(L, std::abs(H.s), ss, rc);
  const int64_t npx = (int64_t)grid_rings(L, ss) * grid_ring_len(L, ss);
  if (dir == 0 || dir == 3) {
    sht_forward(H, f, npx, flm, nb, S, dir == 3);
    if (real) symmetrize_flm(flm, L, (int64_t)L * L, nb, st);
  } else {
    sht_inverse(H, flm, false, f, npx, nb, S, dir == 2);
  }
}

// ---------------------------------------------------------------------------
// heterogeneous batches: every map with its own parameters
// ---------------------------------------------------------------------------

// One pass over the maps on stream st.  Maps with equal parameters (and
// reality) run as one batch on contiguous scratch: inputs gathered and outputs
// scattered with device-to-device copies; a map alone runs in place.
// Reals per element and the used length (in reals) of one f_wav row: the
// transforms advance with the parity-fixed N_j while s2let_n_wav counts N.
int64_t used_wav_reals(const s2let_parameters_t &p, bool real) {
  s2let_parameters_t q = p;
  if (real) {
    q.reality = 1;
    q.spin = 0;
  }
  return make_layout(q, real).woff.back() * (real ? 1 : 2);
}

// Streams of the calling thread for the parameter groups of a multi-map call:
// groups are independent, so they are forked from the caller's stream onto
// these (round robin), run concurrently, and joined back; inside a stream
// capture the fork and join become edges of the graph.  Small band-limits
// leave most of the GPU idle one group at a time (a quadrature launch of a
// map at L = 100 has 16 CTAs).
constexpr int kGroupStreams = 8;
struct GroupStreams {
  cudaStream_t s[kGroupStreams] = {};
  cudaEvent_t fork = nullptr, join[kGroupStreams] = {};
};
GroupStreams &group_streams() {
  static thread_local GroupStreams g;
  if (!g.fork) {
    for (int k = 0; k < kGroupStreams; ++k) {
      S2G_CUDA(cudaStreamCreateWithFlags(&g.s[k], cudaStreamNonBlocking));
      S2G_CUDA(cudaEventCreateWithFlags(&g.join[k], cudaEventDisableTiming));
    }
    S2G_CUDA(cudaEventCreateWithFlags(&g.fork, cudaEventDisableTiming));
  }
  return g;
}

// f32: every map's arrays hold floats (interleaved pairs when complex); they
// are widened into FP64 batch scratch on the way in and rounded on the way out
// (only the used part of f_wav), so every map goes through the scratch.
void multi_pass_group(Op op, const std::vector<int> &g, const s2let_parameters_t *params, const int *real,
                      void *const *px, void *const *wav, void *const *scal, cudaStream_t st, bool f32);

void multi_pass(Op op, int n, const s2let_parameters_t *params, const int *real, void *const *px,
                void *const *wav, void *const *scal, cudaStream_t st, bool f32 = false) {
  std::map<std::string, std::vector<int>> groups;
  for (int k = 0; k < n; ++k) {
    std::string key((const char *)&params[k], sizeof(s2let_parameters_t));
    key.push_back(real[k] ? 1 : 0);
    groups[key].push_back(k);
  }
  const int K = std::min<int>(kGroupStreams, (int)groups.size());
  if (K <= 1) {
    for (auto &kv : groups) multi_pass_group(op, kv.second, params, real, px, wav, scal, st, f32);
    return;
  }
  GroupStreams &gs = group_streams();
  S2G_CUDA(cudaEventRecord(gs.fork, st));
  for (int k = 0; k < K; ++k) S2G_CUDA(cudaStreamWaitEvent(gs.s[k], gs.fork, 0));
  // largest band-limits first, so that the long groups start early
  std::vector<const std::vector<int> *> order;
  for (auto &kv : groups) order.push_back(&kv.second);
  std::stable_sort(order.begin(), order.end(), [&](const std::vector<int> *x, const std::vector<int> *y) {
    return params[(*x)[0]].L > params[(*y)[0]].L;
  });
  for (size_t i = 0; i < order.size(); ++i)
    multi_pass_group(op, *order[i], params, real, px, wav, scal, gs.s[i % K], f32);
  for (int k = 0; k < K; ++k) {
    S2G_CUDA(cudaEventRecord(gs.join[k], gs.s[k]));
    S2G_CUDA(cudaStreamWaitEvent(st, gs.join[k], 0));
  }
}

void multi_pass_group(Op op, const std::vector<int> &g, const s2let_parameters_t *params, const int *real,
                      void *const *px, void *const *wav, void *const *scal, cudaStream_t st, bool f32) {
  {
    const s2let_parameters_t &p = params[g[0]];
    const bool re = real[g[0]] != 0;
    if (g.size() == 1 && !f32) {
      run_directional(op, p, re, px[g[0]], nullptr, wav[g[0]], scal[g[0]], 1, st);
      return;
    }
    const int nb = (int)g.size();
    const size_t esz = re ? sizeof(double) : sizeof(double2);
    const size_t bpx = esz * s2let_n_px(&p), bw = esz * s2let_n_wav(&p), bs = esz * s2let_n_scal(&p);
    const int64_t rpx = (int64_t)(bpx / sizeof(double)), rw = (int64_t)(bw / sizeof(double)),
                  rs = (int64_t)(bs / sizeof(double)), rwu = f32 ? used_wav_reals(p, re) : rw;
    Scratch S(st);
    char *dpx = S.get<char>((int64_t)nb * bpx), *dw = S.get<char>((int64_t)nb * bw),
         *ds = S.get<char>((int64_t)nb * bs);
    const bool fwd = (op == OP_PX2WAV || op == OP_ADJ_PX2WAV);
    for (int i = 0; i < nb; ++i) {
      const int k = g[i];
      if (f32) {
        if (fwd) {
          widen_rows((const float *)px[k], 0, (double *)(dpx + i * bpx), 0, rpx, 1, st);
        } else {
          widen_rows((const float *)wav[k], 0, (double *)(dw + i * bw), 0, rwu, 1, st);
          widen_rows((const float *)scal[k], 0, (double *)(ds + i * bs), 0, rs, 1, st);
        }
      } else if (fwd) {
        S2G_CUDA(cudaMemcpyAsync(dpx + i * bpx, px[k], bpx, cudaMemcpyDeviceToDevice, st));
      } else {
        S2G_CUDA(cudaMemcpyAsync(dw + i * bw, wav[k], bw, cudaMemcpyDeviceToDevice, st));
        S2G_CUDA(cudaMemcpyAsync(ds + i * bs, scal[k], bs, cudaMemcpyDeviceToDevice, st));
      }
    }
    run_directional(op, p, re, dpx, nullptr, dw, ds, nb, st);
    for (int i = 0; i < nb; ++i) {
      const int k = g[i];
      if (f32) {
        if (fwd) {
          narrow_rows((const double *)(dw + i * bw), 0, (float *)wav[k], 0, rwu, 1, st);
          narrow_rows((const double *)(ds + i * bs), 0, (float *)scal[k], 0, rs, 1, st);
        } else {
          narrow_rows((const double *)(dpx + i * bpx), 0, (float *)px[k], 0, rpx, 1, st);
        }
      } else if (fwd) {
        S2G_CUDA(cudaMemcpyAsync(wav[k], dw + i * bw, bw, cudaMemcpyDeviceToDevice, st));
        S2G_CUDA(cudaMemcpyAsync(scal[k], ds + i * bs, bs, cudaMemcpyDeviceToDevice, st));
      } else {
        S2G_CUDA(cudaMemcpyAsync(px[k], dpx + i * bpx, bpx, cudaMemcpyDeviceToDevice, st));
      }
    }
  }
}

// Graphs of repeated heterogeneous batches, keyed by everything the launch
// sequence depends on (operation, parameters, reality, pointers, precision,
// table mode, wavelet kernel).  The first call with a key runs eagerly (it
// builds the plans: device allocation and host synchronisation, which a
// capture cannot contain); the second captures the pass into a CUDA graph; later
// calls replay it.  Plans released => graphs released.
std::mutex g_multi_mu;
std::map<std::string, cudaGraphExec_t> g_multi_graphs;
std::set<std::string> g_multi_seen;

void release_multi_graphs() {
  std::lock_guard<std::mutex> lk(g_multi_mu);
  for (auto &kv : g_multi_graphs) cudaGraphExecDestroy(kv.second);
  g_multi_graphs.clear();
  g_multi_seen.clear();
}

void run_multi(Op op, int n, const s2let_parameters_t *params, const int *real, void *const *px,
               void *const *wav, void *const *scal, bool use_graph, cudaStream_t st, bool f32 = false) {
  S2G_REQUIRE(n >= 0, ERR_INVALID, "negative map count");
  S2G_REQUIRE(n == 0 || (params && real && px && wav && scal), ERR_INVALID, "NULL array");
  for (int k = 0; k < n; ++k) validate(&params[k]);
  if (!use_graph || st == nullptr || timing_enabled()) {
    multi_pass(op, n, params, real, px, wav, scal, st, f32);
    return;
  }
  std::string key;
  auto put = [&key](const void *x, size_t b) { key.append((const char *)x, b); };
  const int op_i = (int)op, kern = current_kernel_type();
  put(&op_i, sizeof op_i);
  put(&n, sizeof n);
  put(params, sizeof(s2let_parameters_t) * n);
  put(real, sizeof(int) * n);
  put(px, sizeof(void *) * n);
  put(wav, sizeof(void *) * n);
  put(scal, sizeof(void *) * n);
  put(&t_precision, sizeof t_precision);
  put(&t_table_mode, sizeof t_table_mode);
  put(&kern, sizeof kern);
  put(&f32, sizeof f32);
  const int tune = autotune_mode();  // tuned launch shapes: a graph of their own
  put(&tune, sizeof tune);
  std::lock_guard<std::mutex> lk(g_multi_mu);
  auto it = g_multi_graphs.find(key);
  if (it != g_multi_graphs.end()) {
    S2G_CUDA(cudaGraphLaunch(it->second, st));
    return;
  }
  if (!g_multi_seen.count(key)) {
    multi_pass(op, n, params, real, px, wav, scal, st, f32);
    g_multi_seen.insert(key);
    return;
  }
  cudaGraph_t graph = nullptr;
  S2G_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  try {
    multi_pass(op, n, params, real, px, wav, scal, st, f32);
  } catch (...) {
    cudaStreamEndCapture(st, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  S2G_CUDA(cudaStreamEndCapture(st, &graph));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  S2G_CUDA(e);
  g_multi_graphs.emplace(key, exec);
  S2G_CUDA(cudaGraphLaunch(exec, st));
}

}  // namespace s2g

// ===========================================================================
// C ABI
// ===========================================================================

using s2g::cplx;

namespace {

int host_directional(const char *fn, s2g::Op op, const s2let_parameters_t *p, bool real, void *px,
                     void *lm, void *wav, void *scal) {
  return s2g::guarded(fn, [&] {
    s2g::validate(p);
    s2g::ensure_device();
    cudaStream_t st = s2g::host_stream();
    s2g::Scratch S(st);
    s2g::Staged io(S);
    const int L = p->L;
    const int64_t npx = s2let_n_px(p), ns = s2let_n_scal(p);
    // the transforms advance scale offsets with N_j; when some N_j < N the end of
    // the s2let_n_wav-sized buffer is never touched (src/c/s2let_analysis.c:340-350),
    // so only the used prefix crosses the bus
    s2let_parameters_t q = *p;
    if (real) {
      q.reality = 1;
      q.spin = 0;
    }
    const int64_t nw = s2g::make_layout(q, real).woff.back();
    const int64_t dd = real ? 1 : 2;  // doubles per sample
    void *dpx = nullptr, *dlm = nullptr, *dwav = nullptr, *dscal = nullptr;
    using namespace s2g;
    const bool px_in = (op == OP_PX2WAV || op == OP_ADJ_PX2WAV);
    const bool px_out = (op == OP_WAV2PX || op == OP_ADJ_WAV2PX);
    const bool lm_in = (op == OP_LM2WAV || op == OP_ADJ_LM2WAV);
    const bool lm_out = (op == OP_WAV2LM || op == OP_ADJ_WAV2LM);
    const bool wav_in = px_out || lm_out;
    if (px_in) dpx = io.in<double>(px, npx * dd);
    if (px_out) dpx = io.out<double>(px, npx * dd);
    if (lm_in) dlm = io.in<double2>(lm, (int64_t)L * L);
    if (lm_out) dlm = io.out<double2>(lm, (int64_t)L * L);
    if (wav_in) {
      dwav = io.in<double>(wav, nw * dd);
      dscal = io.in<double>(scal, ns * dd);
    } else {
      dwav = io.out<double>(wav, nw * dd);
      dscal = io.out<double>(scal, ns * dd);
    }
    run_directional(op, *p, real, dpx, dlm, dwav, dscal, 1, st);
    io.finish();
  });
}

void host_sht(const char *fn, int dir, int L, int spin, bool real, void *f, void *flm, int ss = 0) {
  s2g::guarded(fn, [&] {
    s2g::ensure_device();
    cudaStream_t st = s2g::host_stream();
    s2g::Scratch S(st);
    s2g::Staged io(S);
    const int64_t npx = (int64_t)s2g::grid_rings(L, ss) * s2g::grid_ring_len(L, ss) * (real ? 1 : 2);
    void *df;
    double2 *dlm;
    if (dir == 0 || dir == 3) {
      df = io.in<double>(f, npx);
      dlm = io.out<double2>(flm, (int64_t)L * L);
    } else {
      dlm = io.in<double2>(flm, (int64_t)L * L);
      df = io.out<double>(f, npx);
    }
    s2g::run_sht(dir, L, spin, real, ss, df, dlm, 1, st);
    io.finish();
  });
}

int batch_directional(const char *fn, s2g::Op op, const s2let_parameters_t *p, bool real, void *px,
                      void *wav, void *scal, int nb, void *stream) {
  return s2g::guarded(fn, [&] {
    s2g::validate(p);
    s2g::ensure_device();
    s2g::run_directional(op, *p, real, px, nullptr, wav, scal, nb, (cudaStream_t)stream);
  });
}

// FP32 storage: the batch widened into FP64 device scratch (only the used part
// of each f_wav row), the FP64-storage path at the thread's precision, the
// outputs rounded to FP32.
int batch_directional_f32(const char *fn, s2g::Op op, const s2let_parameters_t *p, bool real, void *px,
                          void *wav, void *scal, int nb, void *stream) {
  return s2g::guarded(fn, [&] {
    using namespace s2g;
    validate(p);
    ensure_device();
    S2G_REQUIRE(nb >= 0, ERR_INVALID, "negative batch size");
    if (nb == 0) return;
    S2G_REQUIRE(px && wav && scal, ERR_INVALID, "NULL buffer");
    cudaStream_t st = (cudaStream_t)stream;
    const int dd = real ? 1 : 2;
    const int64_t npx = s2let_n_px(p) * dd, nw = s2let_n_wav(p) * dd, ns = s2let_n_scal(p) * dd;
    const int64_t nwu = used_wav_reals(*p, real);
    Scratch S(st);
    double *dpx = S.get<double>((int64_t)nb * npx), *dw = S.get<double>((int64_t)nb * nw),
           *ds = S.get<double>((int64_t)nb * ns);
    const bool fwd = (op == OP_PX2WAV || op == OP_ADJ_PX2WAV);
    if (fwd) {
      widen_rows((const float *)px, npx, dpx, npx, npx, nb, st);
    } else {
      widen_rows((const float *)wav, nw, dw, nw, nwu, nb, st);
      widen_rows((const float *)scal, ns, ds, ns, ns, nb, st);
    }
    run_directional(op, *p, real, dpx, nullptr, dw, ds, nb, st);
    if (fwd) {
      narrow_rows(dw, nw, (float *)wav, nw, nwu, nb, st);
      narrow_rows(ds, ns, (float *)scal, ns, ns, nb, st);
    } else {
      narrow_rows(dpx, npx, (float *)px, npx, npx, nb, st);
    }
  });
}

// Host-pointer batches: nb contiguous maps in host memory (the drop-in layout,
// map b at b * the single-map size).  Up to kHostPass maps run as one device
// batch (the Wigner tables streamed once for all of them), and f_wav crosses
// the bus in pieces of one scale for a group of maps on a second stream,
// overlapped with the transforms (WavPipe): analysis copies each piece out as
// soon as it is written, the largest scales first; synthesis queues every
// piece up front and each group's first kernel waits for its piece.  Only the
// used part of each f_wav (the transforms advance with N_j, the buffer is
// sized with N) crosses the bus, as in the drop-in functions.  Synchronous.
constexpr int kHostPass = 32;   // maps per device batch
constexpr int kHostGroups = 4;  // map groups per scale (pieces of at most 8 maps)
// map groups per scale: kHostGroups, or S2LET_GPU_HOST_GROUPS (1-32).
// Pipelined host batches at L=1024 (32 maps per call) measured 238 / 242 / 241
// maps/s with 4 / 8 / 2 groups: within the run-to-run spread.
int host_groups() {
  static const int g = [] {
    const char *e = getenv("S2LET_GPU_HOST_GROUPS");
    const int v = e ? atoi(e) : 0;
    return (v >= 1 && v <= 32) ? v : kHostGroups;
  }();
  return g;
}
int host_pass(int nb) {
  const char *e = getenv("S2LET_GPU_HOST_PASS");
  const int v = e ? atoi(e) : 0;
  const int cap = v > 0 ? v : kHostPass;
  return nb < cap ? nb : cap;
}

int host_batch(const char *fn, s2g::Op op, const s2let_parameters_t *p, bool real, void *px, void *wav,
               void *scal, int nb) {
  return s2g::guarded(fn, [&] {
    using namespace s2g;
    validate(p);
    ensure_device();
    S2G_REQUIRE(nb >= 0, ERR_INVALID, "negative batch size");
    if (nb == 0) return;
    S2G_REQUIRE(px && wav && scal, ERR_INVALID, "NULL buffer");
    // the copy stream has the highest priority: its copy kernels take SM
    // slots as soon as the transforms free some
    static thread_local cudaStream_t sts[2] = {nullptr, nullptr};
    if (!sts[0]) S2G_CUDA(cudaStreamCreateWithFlags(&sts[0], cudaStreamNonBlocking));
    if (!sts[1]) {
      int least = 0, greatest = 0;
      S2G_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      S2G_CUDA(cudaStreamCreateWithPriority(&sts[1], cudaStreamNonBlocking, greatest));
    }
    cudaStream_t st = sts[0], cs = sts[1];
    const size_t esz = real ? sizeof(double) : sizeof(double2);
    s2let_parameters_t q = *p;
    if (real) {
      q.reality = 1;
      q.spin = 0;
    }
    const int64_t npx = s2let_n_px(p), nw = s2let_n_wav(p), ns = s2let_n_scal(p);
    const int64_t nwu = make_layout(q, real).woff.back();  // used part of one f_wav
    const bool fwd = (op == OP_PX2WAV || op == OP_ADJ_PX2WAV);
    const WavPlan &P = directional_plan(*p, real);
    char *hpx = (char *)px, *hw = (char *)wav, *hs = (char *)scal;
    const int pass = host_pass(nb);
    for (int c0 = 0; c0 < nb; c0 += pass) {
      const int n = std::min(pass, nb - c0);
      Scratch S(st);
      char *dpx = S.get<char>((int64_t)n * npx * esz), *dw = S.get<char>((int64_t)n * nw * esz),
           *ds = S.get<char>((int64_t)n * ns * esz);
      // both streams idle before the buffers are released, also on an error
      struct Drain {
        cudaStream_t a, b;
        ~Drain() {
          cudaStreamSynchronize(a);
          cudaStreamSynchronize(b);
        }
      } drain{cs, st};
      WavPipe pipe;
      pipe.cs = cs;
      pipe.host = hw + (size_t)c0 * nw * esz;
      pipe.hstride = nw;
      pipe.esz = esz;
      const int ngrp = host_groups();
      pipe.group = std::max(1, std::min(8, (n + ngrp - 1) / ngrp));
      for (size_t k = 0; k < P.sc.size(); ++k)
        pipe.seglen[P.sc[k].woff] = (k + 1 < P.sc.size() ? P.sc[k + 1].woff : nwu) - P.sc[k].woff;
      // the copy stream uses the new buffers only after their allocation on st
      cudaEvent_t e0 = pipe.event();
      S2G_CUDA(cudaEventRecord(e0, st));
      S2G_CUDA(cudaStreamWaitEvent(cs, e0, 0));
      if (fwd) {
        copy_async(dpx, 0, hpx + (size_t)c0 * npx * esz, 0, (size_t)n * npx * esz, 1, cudaMemcpyHostToDevice, st);
        run_plan(op, P, dpx, nullptr, dw, nw, ds, ns, n, st, false, &pipe);
        copy_async(hs + (size_t)c0 * ns * esz, 0, ds, 0, (size_t)n * ns * esz, 1, cudaMemcpyDeviceToHost, st);
      } else {
        copy_async(ds, 0, hs + (size_t)c0 * ns * esz, 0, (size_t)n * ns * esz, 1, cudaMemcpyHostToDevice, st);
        for (const auto &pk : table_passes(P, true))  // in the order the synthesis reads them
          for (size_t k = pk.first; k < pk.second; ++k) {
            const Scale &sd = P.sc[k];
            if (rings_on_n(P, sd)) {
              for (int b0 = 0; b0 < n; b0 += pipe.group) pipe.in(dw, nw, sd.woff, b0, std::min(pipe.group, n - b0));
            } else {
              pipe.in(dw, nw, sd.woff, 0, n);
            }
          }
        run_plan(op, P, dpx, nullptr, dw, nw, ds, ns, n, st, false, &pipe);
        copy_async(hpx + (size_t)c0 * npx * esz, 0, dpx, 0, (size_t)n * npx * esz, 1, cudaMemcpyDeviceToHost, st);
      }
    }
  });
}

// ---- axisymmetric pixel-space transforms (src/c/s2let_transform_axisym_mw.c:124-1171)
void host_axisym(const char *fn, s2g::Op op, const s2let_parameters_t *p, bool real, bool multires,
                 void *f, void *wav, void *scal) {
  s2g::guarded(fn, [&] {
    S2G_REQUIRE(p != nullptr, s2g::ERR_INVALID, "parameters is NULL");
    s2let_parameters_t q = *p;
    q.spin = 0;  // the axisymmetric transforms are spin 0 (src/c/s2let_transform_axisym_mw.c:132)
    q.N = 1;
    s2g::validate(&q, false);
    s2g::ensure_device();
    cudaStream_t st = s2g::host_stream();
    s2g::Scratch S(st);
    s2g::Staged io(S);
    const s2g::WavPlan &P = s2g::axisym_plan(q, real, multires);
    const int L = q.L;
    const int64_t npx = (int64_t)L * (2 * L - 1);
    int64_t nw = 0;
    for (const auto &sd : P.sc) nw += (int64_t)sd.bl * (2 * sd.bl - 1);
    const int64_t ns = (int64_t)P.bl_scal * (2 * P.bl_scal - 1);
    const int64_t dd = real ? 1 : 2;
    using namespace s2g;
    void *dpx, *dwav, *dscal;
    if (op == OP_PX2WAV || op == OP_ADJ_PX2WAV) {
      dpx = io.in<double>(f, npx * dd);
      dwav = io.out<double>(wav, nw * dd);
      dscal = io.out<double>(scal, ns * dd);
    } else {
      dpx = io.out<double>(f, npx * dd);
      dwav = io.in<double>(wav, nw * dd);
      dscal = io.in<double>(scal, ns * dd);
    }
    s2g::run_plan(op, P, dpx, nullptr, dwav, nw, dscal, ns, 1, st);
    io.finish();
  });
}

// ---- manual tilings (src/c/s2let_analysis.c:188-276 and the three siblings)
void host_manual(const char *fn, s2g::Op op, cplx *flm, cplx *f_wav, cplx *f_scal, const double *scal_l,
                 const cplx *wav_lm, int scal_bl, const int *wav_bl, int J, int L, int spin, int N) {
  s2g::guarded(fn, [&] {
    S2G_REQUIRE(L >= 1 && N >= 1 && J >= 0 && std::abs(spin) < L, s2g::ERR_INVALID, "bad manual parameters");
    S2G_REQUIRE(scal_l && wav_lm && wav_bl, s2g::ERR_INVALID, "NULL tiling array");
    s2g::ensure_device();
    using namespace s2g;
    s2g::PlanSpec ps;
    ps.L = L;
    ps.spin = spin;
    ps.real = false;
    ps.bl_scal = std::min(scal_bl, L);
    ps.scal_lmin = std::abs(spin);
    int64_t off = 0;
    for (int j = 0; j <= J; ++j) {
      const int bl = std::min(wav_bl[j], L);
      int Nj = std::min(N, bl);
      Nj += (Nj + N) % 2;
      ps.jrow.push_back(j);
      ps.bl.push_back(bl);
      ps.Nj.push_back(Nj);
      ps.woff.push_back(off);
      off += (int64_t)(2 * Nj - 1) * bl * (2 * bl - 1);
    }
    ps.psi = wav_lm;
    ps.phi = scal_l;
    // the reference's adjoint manual paths multiply by conj(psi) / psi where the
    // exact adjoint would use psi / conj(psi); reproduced as specified there
    // (src/c/s2let_analysis_adjoint.c:278, src/c/s2let_synthesis_adjoint.c:266)
    ps.split_conj = (op == OP_LM2WAV);
    ps.merge_conj = (op == OP_ADJ_WAV2LM);
    auto P = s2g::build_plan(ps);
    if (op == OP_ADJ_LM2WAV) {  // src/c/s2let_synthesis_adjoint.c:215-218
      printf("J = %i\n", J);
      printf("B = %g\n", pow(L, 1.0 / (float)(J + 2)));
      printf("N = %i\n", N);
      printf("L = %i\n", L);
      fflush(stdout);
    }
    cudaStream_t st = s2g::host_stream();
    {
      s2g::Scratch S(st);
      s2g::Staged io(S);
      const int64_t ns = (int64_t)ps.bl_scal * (2 * ps.bl_scal - 1);
      double2 *dlm, *dw, *dsc;
      if (op == OP_LM2WAV || op == OP_ADJ_LM2WAV) {
        dlm = io.in<double2>(flm, (int64_t)L * L);
        dw = io.out<double2>(f_wav, off);
        dsc = io.out<double2>(f_scal, ns);
      } else {  // these two accumulate into flm (src/c/s2let_synthesis.c:254,281)
        dlm = io.inout<double2>(flm, (int64_t)L * L);
        dw = io.in<double2>(f_wav, off);
        dsc = io.in<double2>(f_scal, ns);
      }
      s2g::run_plan(op, *P, nullptr, dlm, dw, off, dsc, ns, 1, st, true);
      io.finish();
    }
    P->release();
  });
}

}  // namespace

extern "C" {

int s2let_gpu_last_error(void) { return s2g::t_status; }
const char *s2let_gpu_last_error_string(void) { return s2g::t_message.c_str(); }
int s2let_gpu_set_precision(int mode) {
  if (mode != 0 && mode != 1) {
    s2g::set_status(s2g::ERR_INVALID, "precision mode must be 0 (FP64) or 1 (mixed)");
    return s2g::ERR_INVALID;
  }
  s2g::t_precision = mode;
  return 0;
}
int s2let_gpu_get_precision(void) { return s2g::t_precision; }
int s2let_gpu_set_table_mode(int mode) {
  if (mode < 0 || mode > 2) {
    s2g::set_status(s2g::ERR_INVALID, "s2let_gpu_set_table_mode: mode must be 0, 1 or 2");
    s2g::report_failure();
    return s2g::ERR_INVALID;
  }
  s2g::t_table_mode = mode;
  return 0;
}
int s2let_gpu_get_table_mode(void) { return s2g::t_table_mode; }
int s2let_gpu_bind_device(int device) {
  const int st = s2g::bind_device(device);
  if (st != s2g::OK) {
    s2g::set_status(st, device < 0 ? "s2let_gpu_bind_device: negative device ordinal"
                                   : "s2let_gpu_bind_device: the library already serves CUDA device " +
                                         std::to_string(s2g::g_bound_device.load()) + " in this process");
    s2g::report_failure();
  }
  return st;
}
int s2let_gpu_bound_device(void) { return s2g::g_bound_device.load(); }
void s2let_gpu_release_plans(void) {
  s2g::guarded("s2let_gpu_release_plans", [] {
    {
      std::lock_guard<std::mutex> lk(s2g::g_plan_mu);
      cudaDeviceSynchronize();
      for (auto &kv : s2g::g_plans) kv.second->release();
      s2g::g_plans.clear();
    }
    s2g::release_multi_graphs();
    s2g::release_sliced_tables();
    s2g::release_df_tables();
    s2g::release_plans();
  });
}
size_t s2let_gpu_plan_bytes(void) {
  return s2g::plan_bytes() + s2g::sliced_table_bytes() + s2g::df_table_bytes();
}
int s2let_gpu_set_split_tables(int on) {
  if (on != 0 && on != 1) {
    s2g::set_status(s2g::ERR_INVALID, "s2let_gpu_set_split_tables: 0 or 1");
    return s2g::ERR_INVALID;
  }
  s2g::set_split_tables(on);
  return 0;
}
int s2let_gpu_get_split_tables(void) { return s2g::get_split_tables(); }
int s2let_gpu_set_df_max_maps(int maps) {
  if (maps < 0 || maps > 4) {
    s2g::set_status(s2g::ERR_INVALID, "s2let_gpu_set_df_max_maps: 0 to 4 maps");
    return s2g::ERR_INVALID;
  }
  s2g::set_df_max_maps(maps);
  return 0;
}
int s2let_gpu_get_df_max_maps(void) { return s2g::get_df_max_maps(); }
int s2let_gpu_device_fault(void) {
  int v = 0;
  s2g::guarded("s2let_gpu_device_fault", [&] { v = s2g::mixed_error_flag_read_and_clear(); });
  return v;
}
uint64_t s2let_gpu_launch_count(void) { return s2g::g_launches.load(); }

// ---- pixel-space directional transforms
void s2let_analysis_px2wav(cplx *f_wav, cplx *f_scal, const cplx *f, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_PX2WAV, p, false, (void *)f, nullptr, f_wav, f_scal);
}
void s2let_analysis_px2wav_real(double *f_wav, double *f_scal, const double *f, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_PX2WAV, p, true, (void *)f, nullptr, f_wav, f_scal);
}
void s2let_synthesis_wav2px(cplx *f, const cplx *f_wav, const cplx *f_scal, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_WAV2PX, p, false, f, nullptr, (void *)f_wav, (void *)f_scal);
}
void s2let_synthesis_wav2px_real(double *f, const double *f_wav, const double *f_scal, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_WAV2PX, p, true, f, nullptr, (void *)f_wav, (void *)f_scal);
}
void s2let_analysis_adjoint_wav2px(cplx *f, const cplx *f_wav, const cplx *f_scal, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_WAV2PX, p, false, f, nullptr, (void *)f_wav, (void *)f_scal);
}
void s2let_analysis_adjoint_wav2px_real(double *f, const double *f_wav, const double *f_scal,
                                        const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_WAV2PX, p, true, f, nullptr, (void *)f_wav, (void *)f_scal);
}
void s2let_synthesis_adjoint_px2wav(cplx *f_wav, cplx *f_scal, const cplx *f, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_PX2WAV, p, false, (void *)f, nullptr, f_wav, f_scal);
}
void s2let_synthesis_adjoint_px2wav_real(double *f_wav, double *f_scal, const double *f,
                                         const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_PX2WAV, p, true, (void *)f, nullptr, f_wav, f_scal);
}

// ---- harmonic-space directional transforms
void s2let_analysis_lm2wav(cplx *f_wav, cplx *f_scal, const cplx *flm, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_LM2WAV, p, false, nullptr, (void *)flm, f_wav, f_scal);
}
void s2let_analysis_lm2wav_real(double *f_wav, double *f_scal, const cplx *flm, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_LM2WAV, p, true, nullptr, (void *)flm, f_wav, f_scal);
}
void s2let_synthesis_wav2lm(cplx *flm, const cplx *f_wav, const cplx *f_scal, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_WAV2LM, p, false, nullptr, flm, (void *)f_wav, (void *)f_scal);
}
void s2let_synthesis_wav2lm_real(cplx *flm, const double *f_wav, const double *f_scal, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_WAV2LM, p, true, nullptr, flm, (void *)f_wav, (void *)f_scal);
}
void s2let_analysis_adjoint_wav2lm(cplx *flm, const cplx *f_wav, const cplx *f_scal, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_WAV2LM, p, false, nullptr, flm, (void *)f_wav, (void *)f_scal);
}
void s2let_analysis_adjoint_wav2lm_real(cplx *flm, const double *f_wav, const double *f_scal,
                                        const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_WAV2LM, p, true, nullptr, flm, (void *)f_wav, (void *)f_scal);
}
void s2let_synthesis_adjoint_lm2wav(cplx *f_wav, cplx *f_scal, const cplx *flm, const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_LM2WAV, p, false, nullptr, (void *)flm, f_wav, f_scal);
}
void s2let_synthesis_adjoint_lm2wav_real(double *f_wav, double *f_scal, const cplx *flm,
                                         const s2let_parameters_t *p) {
  host_directional(__func__, s2g::OP_ADJ_LM2WAV, p, true, nullptr, (void *)flm, f_wav, f_scal);
}

// ---- manual tilings
void s2let_analysis_lm2wav_manual(cplx *f_wav, cplx *f_scal, const cplx *flm, const double *scal_l,
                                  const cplx *wav_lm, const int scal_bandlimit, const int *wav_bandlimits,
                                  int J, int L, int spin, int N) {
  host_manual(__func__, s2g::OP_LM2WAV, (cplx *)flm, f_wav, f_scal, scal_l, wav_lm, scal_bandlimit,
              wav_bandlimits, J, L, spin, N);
}
void s2let_synthesis_wav2lm_manual(cplx *flm, const cplx *f_wav, const cplx *f_scal, const double *scal_l,
                                   const cplx *wav_lm, const int scal_bandlimit, const int *wav_bandlimits,
                                   int J, int L, int spin, int N) {
  host_manual(__func__, s2g::OP_WAV2LM, flm, (cplx *)f_wav, (cplx *)f_scal, scal_l, wav_lm, scal_bandlimit,
              wav_bandlimits, J, L, spin, N);
}
void s2let_analysis_adjoint_wav2lm_manual(cplx *flm, const cplx *f_wav, const cplx *f_scal,
                                          const double *scal_l, const cplx *wav_lm, const int scal_bandlimit,
                                          const int *wav_bandlimits, int J, int L, int spin, int N) {
  host_manual(__func__, s2g::OP_ADJ_WAV2LM, flm, (cplx *)f_wav, (cplx *)f_scal, scal_l, wav_lm,
              scal_bandlimit, wav_bandlimits, J, L, spin, N);
}
void s2let_synthesis_adjoint_lm2wav_manual(cplx *f_wav, cplx *f_scal, const cplx *flm, const double *scal_l,
                                           const cplx *wav_lm, const int scal_bandlimit,
                                           const int *wav_bandlimits, int J, int L, int spin, int N) {
  host_manual(__func__, s2g::OP_ADJ_LM2WAV, (cplx *)flm, f_wav, f_scal, scal_l, wav_lm, scal_bandlimit,
              wav_bandlimits, J, L, spin, N);
}

// ---- axisymmetric pixel-space transforms
#define S2G_AXI(name, op, mr, re, TA, TB, TC)                                                     \
  void name(TA *a, TB *b, TC *c, const s2let_parameters_t *p) {                                  \
    if (op == s2g::OP_PX2WAV || op == s2g::OP_ADJ_PX2WAV)                                        \
      host_axisym(#name, op, p, re, mr, (void *)c, (void *)a, (void *)b);                       \
    else                                                                                         \
      host_axisym(#name, op, p, re, mr, (void *)a, (void *)b, (void *)c);                       \
  }
// analysis / synthesis-adjoint: (f_wav, f_scal, f);  synthesis / analysis-adjoint: (f, f_wav, f_scal)
S2G_AXI(s2let_transform_axisym_wav_analysis_mw, s2g::OP_PX2WAV, false, false, cplx, cplx, const cplx)
S2G_AXI(s2let_transform_axisym_wav_analysis_mw_multires, s2g::OP_PX2WAV, true, false, cplx, cplx, const cplx)
S2G_AXI(s2let_transform_axisym_wav_analysis_mw_real, s2g::OP_PX2WAV, false, true, double, double, const double)
S2G_AXI(s2let_transform_axisym_wav_analysis_mw_multires_real, s2g::OP_PX2WAV, true, true, double, double,
        const double)
S2G_AXI(s2let_transform_axisym_wav_synthesis_adjoint_mw, s2g::OP_ADJ_PX2WAV, false, false, cplx, cplx, const cplx)
S2G_AXI(s2let_transform_axisym_wav_synthesis_adjoint_mw_multires, s2g::OP_ADJ_PX2WAV, true, false, cplx, cplx,
        const cplx)
S2G_AXI(s2let_transform_axisym_wav_synthesis_adjoint_mw_real, s2g::OP_ADJ_PX2WAV, false, true, double, double,
        const double)
S2G_AXI(s2let_transform_axisym_wav_synthesis_adjoint_mw_multires_real, s2g::OP_ADJ_PX2WAV, true, true, double,
        double, const double)
S2G_AXI(s2let_transform_axisym_wav_synthesis_mw, s2g::OP_WAV2PX, false, false, cplx, const cplx, const cplx)
S2G_AXI(s2let_transform_axisym_wav_synthesis_mw_multires, s2g::OP_WAV2PX, true, false, cplx, const cplx, const cplx)
S2G_AXI(s2let_transform_axisym_wav_synthesis_mw_real, s2g::OP_WAV2PX, false, true, double, const double,
        const double)
S2G_AXI(s2let_transform_axisym_wav_synthesis_mw_multires_real, s2g::OP_WAV2PX, true, true, double, const double,
        const double)
S2G_AXI(s2let_transform_axisym_wav_analysis_adjoint_mw, s2g::OP_ADJ_WAV2PX, false, false, cplx, const cplx,
        const cplx)
S2G_AXI(s2let_transform_axisym_wav_analysis_adjoint_mw_multires, s2g::OP_ADJ_WAV2PX, true, false, cplx,
        const cplx, const cplx)
S2G_AXI(s2let_transform_axisym_wav_analysis_adjoint_mw_real, s2g::OP_ADJ_WAV2PX, false, true, double,
        const double, const double)
S2G_AXI(s2let_transform_axisym_wav_analysis_adjoint_mw_multires_real, s2g::OP_ADJ_WAV2PX, true, true, double,
        const double, const double)
#undef S2G_AXI

// ---- plain MW spherical-harmonic transforms (src/c/s2let_mw.c:21-94)
void s2let_mw_alm2map(cplx *f, const cplx *flm, int L, int spin) { host_sht(__func__, 1, L, spin, false, f, (void *)flm); }
void s2let_mw_map2alm(cplx *flm, const cplx *f, int L, int spin) { host_sht(__func__, 0, L, spin, false, (void *)f, flm); }
void s2let_mw_alm2map_real(double *f, const cplx *flm, int L) { host_sht(__func__, 1, L, 0, true, f, (void *)flm); }
void s2let_mw_map2alm_real(cplx *flm, const double *f, int L) { host_sht(__func__, 0, L, 0, true, (void *)f, flm); }
double s2let_mw_power(cplx *f, int L) {
  std::vector<cplx> flm((size_t)L * L);
  s2let_mw_map2alm(flm.data(), f, L, 0);
  return s2let_lm_power(flm.data(), L);
}
double s2let_mw_power_real(double *f, int L) {
  std::vector<cplx> flm((size_t)L * L);
  s2let_mw_map2alm_real(flm.data(), f, L);
  return s2let_lm_power(flm.data(), L);
}
// Adjoints of the plain transforms (SSHT adjoints that S2LET uses internally).
void s2let_gpu_mw_adjoint_map2alm(cplx *f, const cplx *flm, int L, int spin) {
  host_sht(__func__, 2, L, spin, false, f, (void *)flm);
}
void s2let_gpu_mw_adjoint_alm2map(cplx *flm, const cplx *f, int L, int spin) {
  host_sht(__func__, 3, L, spin, false, (void *)f, flm);
}
// Plain transforms on either sampling (the SSHT entry points that the wavelet
// transforms call, MW or MWSS), host buffers.
int s2let_gpu_sht(int dir, int sampling_scheme, int L, int spin, int real, void *f, void *flm) {
  if (sampling_scheme != S2LET_SAMPLING_MW && sampling_scheme != S2LET_SAMPLING_MW_SS) {
    s2g::set_status(s2g::ERR_UNSUPPORTED, "s2let_gpu_sht: unknown sampling scheme");
    s2g::report_failure();
    return s2g::ERR_UNSUPPORTED;
  }
  if (dir < 0 || dir > 3 || f == nullptr || flm == nullptr) {
    s2g::set_status(s2g::ERR_INVALID, "s2let_gpu_sht: bad direction or NULL buffer");
    s2g::report_failure();
    return s2g::ERR_INVALID;
  }
  host_sht(__func__, dir, L, spin, real != 0, f, flm, sampling_scheme == S2LET_SAMPLING_MW_SS);
  return s2g::last_status();
}

// ---- host-pointer batches (drop-in layout, nbatch maps per call)
int s2let_gpu_analysis_px2wav_real_host_batch(double *f_wav, double *f_scal, const double *f, int nb,
                                              const s2let_parameters_t *p) {
  return host_batch(__func__, s2g::OP_PX2WAV, p, true, (void *)f, f_wav, f_scal, nb);
}
int s2let_gpu_synthesis_wav2px_real_host_batch(double *f, const double *f_wav, const double *f_scal, int nb,
                                               const s2let_parameters_t *p) {
  return host_batch(__func__, s2g::OP_WAV2PX, p, true, f, (void *)f_wav, (void *)f_scal, nb);
}
int s2let_gpu_analysis_px2wav_host_batch(void *f_wav, void *f_scal, const void *f, int nb,
                                         const s2let_parameters_t *p) {
  return host_batch(__func__, s2g::OP_PX2WAV, p, false, (void *)f, f_wav, f_scal, nb);
}
int s2let_gpu_synthesis_wav2px_host_batch(void *f, const void *f_wav, const void *f_scal, int nb,
                                          const s2let_parameters_t *p) {
  return host_batch(__func__, s2g::OP_WAV2PX, p, false, f, (void *)f_wav, (void *)f_scal, nb);
}

// ---- heterogeneous batches (device pointers, per-map parameters)
int s2let_gpu_px2wav_multi(void *const *f_wav, void *const *f_scal, void *const *f,
                           const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                           void *stream) {
  return s2g::guarded(__func__, [&] {
    s2g::ensure_device();
    s2g::run_multi(s2g::OP_PX2WAV, nmaps, params, real, f, f_wav, f_scal, use_graph != 0, (cudaStream_t)stream);
  });
}
int s2let_gpu_wav2px_multi(void *const *f, void *const *f_wav, void *const *f_scal,
                           const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                           void *stream) {
  return s2g::guarded(__func__, [&] {
    s2g::ensure_device();
    s2g::run_multi(s2g::OP_WAV2PX, nmaps, params, real, f, f_wav, f_scal, use_graph != 0, (cudaStream_t)stream);
  });
}

// ---- batched device-pointer extensions
int s2let_gpu_analysis_px2wav_real_batch(double *f_wav, double *f_scal, const double *f, int nb,
                                         const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_PX2WAV, p, true, (void *)f, f_wav, f_scal, nb, stream);
}
int s2let_gpu_synthesis_wav2px_real_batch(double *f, const double *f_wav, const double *f_scal, int nb,
                                          const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_WAV2PX, p, true, f, (void *)f_wav, (void *)f_scal, nb, stream);
}
int s2let_gpu_analysis_px2wav_batch(void *f_wav, void *f_scal, const void *f, int nb,
                                    const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_PX2WAV, p, false, (void *)f, f_wav, f_scal, nb, stream);
}
int s2let_gpu_synthesis_wav2px_batch(void *f, const void *f_wav, const void *f_scal, int nb,
                                     const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_WAV2PX, p, false, f, (void *)f_wav, (void *)f_scal, nb, stream);
}
int s2let_gpu_analysis_adjoint_wav2px_real_batch(double *f, const double *f_wav, const double *f_scal, int nb,
                                                 const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_ADJ_WAV2PX, p, true, f, (void *)f_wav, (void *)f_scal, nb, stream);
}
int s2let_gpu_synthesis_adjoint_px2wav_real_batch(double *f_wav, double *f_scal, const double *f, int nb,
                                                  const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_ADJ_PX2WAV, p, true, (void *)f, f_wav, f_scal, nb, stream);
}
int s2let_gpu_analysis_adjoint_wav2px_batch(void *f, const void *f_wav, const void *f_scal, int nb,
                                            const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_ADJ_WAV2PX, p, false, f, (void *)f_wav, (void *)f_scal, nb, stream);
}
int s2let_gpu_synthesis_adjoint_px2wav_batch(void *f_wav, void *f_scal, const void *f, int nb,
                                             const s2let_parameters_t *p, void *stream) {
  return batch_directional(__func__, s2g::OP_ADJ_PX2WAV, p, false, (void *)f, f_wav, f_scal, nb, stream);
}

// ---- FP32 storage (batched device pointers)
int s2let_gpu_analysis_px2wav_real_batch_f32(float *f_wav, float *f_scal, const float *f, int nb,
                                             const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_PX2WAV, p, true, (void *)f, f_wav, f_scal, nb, stream);
}
int s2let_gpu_synthesis_wav2px_real_batch_f32(float *f, const float *f_wav, const float *f_scal, int nb,
                                              const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_WAV2PX, p, true, f, (void *)f_wav, (void *)f_scal, nb, stream);
}
int s2let_gpu_analysis_px2wav_batch_f32(void *f_wav, void *f_scal, const void *f, int nb,
                                        const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_PX2WAV, p, false, (void *)f, f_wav, f_scal, nb, stream);
}
int s2let_gpu_synthesis_wav2px_batch_f32(void *f, const void *f_wav, const void *f_scal, int nb,
                                         const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_WAV2PX, p, false, f, (void *)f_wav, (void *)f_scal, nb, stream);
}
int s2let_gpu_analysis_adjoint_wav2px_real_batch_f32(float *f, const float *f_wav, const float *f_scal, int nb,
                                                     const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_ADJ_WAV2PX, p, true, f, (void *)f_wav, (void *)f_scal, nb,
                               stream);
}
int s2let_gpu_synthesis_adjoint_px2wav_real_batch_f32(float *f_wav, float *f_scal, const float *f, int nb,
                                                      const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_ADJ_PX2WAV, p, true, (void *)f, f_wav, f_scal, nb, stream);
}
int s2let_gpu_analysis_adjoint_wav2px_batch_f32(void *f, const void *f_wav, const void *f_scal, int nb,
                                                const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_ADJ_WAV2PX, p, false, f, (void *)f_wav, (void *)f_scal, nb,
                               stream);
}
int s2let_gpu_synthesis_adjoint_px2wav_batch_f32(void *f_wav, void *f_scal, const void *f, int nb,
                                                 const s2let_parameters_t *p, void *stream) {
  return batch_directional_f32(__func__, s2g::OP_ADJ_PX2WAV, p, false, (void *)f, f_wav, f_scal, nb, stream);
}
int s2let_gpu_px2wav_multi_f32(void *const *f_wav, void *const *f_scal, void *const *f,
                               const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                               void *stream) {
  return s2g::guarded(__func__, [&] {
    s2g::ensure_device();
    s2g::run_multi(s2g::OP_PX2WAV, nmaps, params, real, f, f_wav, f_scal, use_graph != 0, (cudaStream_t)stream,
                   true);
  });
}
int s2let_gpu_wav2px_multi_f32(void *const *f, void *const *f_wav, void *const *f_scal,
                               const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                               void *stream) {
  return s2g::guarded(__func__, [&] {
    s2g::ensure_device();
    s2g::run_multi(s2g::OP_WAV2PX, nmaps, params, real, f, f_wav, f_scal, use_graph != 0, (cudaStream_t)stream,
                   true);
  });
}

}  // extern "C"
