// C ABI: harmonic-space tiling multiplies on the reference's layouts
//   s2let_analysis_lm2lmn(_real)            src/c/s2let_analysis.c:28-161
//   s2let_synthesis_lmn2lm(_real)           src/c/s2let_synthesis.c:25-175
//   s2let_analysis_adjoint_lmn2lm(_real)    src/c/s2let_analysis_adjoint.c:25-175
//   s2let_synthesis_adjoint_lm2lmn(_real)   src/c/s2let_synthesis_adjoint.c:28-175
//   s2let_transform_axisym_lm_wav_*         src/c/s2let_transform_axisym_lm.c:133-308
//   s2let_transform_axisym_wav_hardthreshold_*  src/c/s2let_transform_axisym_mw.c:1183-1225
// Each stages the caller's host arrays on the device, runs one streaming kernel
// and copies the results back.  Output entries that the reference does not
// write keep the caller's values (outputs are staged in and out).
#include <vector>

#include "common.h"
#include "host_layer.h"
#include "kernels.h"
#include "runtime.h"

using s2g::cplx;

namespace {

// Scale offsets inside f_wav_lmn.  The storage sizes follow p.reality even for
// the _real functions, as fill_so3_parameters does (include/s2let/s2let_so3.h:24-42);
// `real` only selects the n >= 0 index map.
std::vector<s2g::LmnScale> lmn_scales(const s2let_parameters_t &p, bool real, int *nmax, int64_t *extent) {
  const s2g::Layout g = s2g::make_layout(p, real);
  std::vector<s2g::LmnScale> v;
  *nmax = 1;
  int64_t off = 0;
  for (int k = 0; k < g.nscale(); ++k) {
    v.push_back(s2g::LmnScale{g.j[k], g.bl[k], g.Nj[k], off});
    s2g::SO3Shape s = g.so3[k];
    s.reality = p.reality;
    off += s.flmn_size();
    *nmax = std::max(*nmax, g.Nj[k]);
  }
  *extent = off;
  return v;
}

// split: flm -> (f_wav_lmn, f_scal_lm);  mode 0 analysis, 1 synthesis adjoint
void lm_split(const char *fn, int mode, cplx *flmn, cplx *fscal, const cplx *flm, const cplx *psi,
              const double *phi, const s2let_parameters_t *p, bool real) {
  s2g::guarded(fn, [&] {
    s2g::validate(p, false);
    s2g::ensure_device();
    cudaStream_t st = s2g::host_stream();
    s2g::Scratch S(st);
    s2g::Staged io(S);
    const int L = p->L, J = s2g::j_max(*p);
    int nmax;
    int64_t extent;
    auto sc = lmn_scales(*p, real, &nmax, &extent);
    const int bs = p->upsample ? L : std::min(s2g::bandlimit(p->J_min - 1, *p), L);
    double2 *d_flmn = io.inout<double2>(flmn, extent);
    double2 *d_fs = io.inout<double2>(fscal, (int64_t)bs * bs);
    const double2 *d_flm = io.in<double2>(flm, (int64_t)L * L);
    const double2 *d_psi = io.in<double2>(psi, (int64_t)(J + 1) * L * L);
    const double *d_phi = io.in<double>(phi, L);
    s2g::LmnScale *d_sc = io.in<s2g::LmnScale>(sc.data(), (int64_t)sc.size());
    s2g::lmn_split(d_flmn, d_fs, d_flm, d_psi, d_phi, d_sc, (int)sc.size(), nmax, L, bs, real ? 0 : p->spin,
                   real, mode, st);
    io.finish();
  });
}

// merge: (f_wav_lmn, f_scal_lm) -> flm;  mode 0 synthesis, 1 analysis adjoint
void lm_merge(const char *fn, int mode, cplx *flm, const cplx *flmn, const cplx *fscal, const cplx *psi,
              const double *phi, const s2let_parameters_t *p, bool real) {
  s2g::guarded(fn, [&] {
    s2g::validate(p, false);
    s2g::ensure_device();
    cudaStream_t st = s2g::host_stream();
    s2g::Scratch S(st);
    s2g::Staged io(S);
    const int L = p->L, J = s2g::j_max(*p);
    int nmax;
    int64_t extent;
    auto sc = lmn_scales(*p, real, &nmax, &extent);
    const int bs = p->upsample ? L : std::min(s2g::bandlimit(p->J_min - 1, *p), L);
    double2 *d_flm = io.out<double2>(flm, (int64_t)L * L);
    const double2 *d_flmn = io.in<double2>(flmn, extent);
    const double2 *d_fs = io.in<double2>(fscal, (int64_t)bs * bs);
    const double2 *d_psi = io.in<double2>(psi, (int64_t)(J + 1) * L * L);
    const double *d_phi = io.in<double>(phi, L);
    s2g::LmnScale *d_sc = io.in<s2g::LmnScale>(sc.data(), (int64_t)sc.size());
    s2g::lmn_merge(d_flm, d_flmn, d_fs, d_psi, d_phi, d_sc, (int)sc.size(), L, bs, real ? 0 : p->spin, real,
                   mode, st);
    io.finish();
  });
}

void axisym_lm_call(const char *fn, bool synth, bool multires, cplx *flm, cplx *fwav, cplx *fscal,
                    const double *wav_lm, const double *scal_lm, const s2let_parameters_t *p) {
  s2g::guarded(fn, [&] {
    S2G_REQUIRE(p != nullptr, s2g::ERR_INVALID, "parameters is NULL");
    s2let_parameters_t q = *p;
    q.N = 1;
    q.spin = 0;
    s2g::validate(&q, false);
    s2g::ensure_device();
    cudaStream_t st = s2g::host_stream();
    s2g::Scratch S(st);
    s2g::Staged io(S);
    const int L = p->L, J = s2g::j_max(*p);
    std::vector<int> bl;
    std::vector<int64_t> off;
    int64_t tot = 0;
    for (int j = p->J_min; j <= J; ++j) {
      const int b = multires ? std::min(s2g::bandlimit(j, *p), L) : L;
      bl.push_back(b);
      off.push_back(tot);
      tot += (int64_t)b * b;
    }
    const int bs = multires ? std::min(s2g::bandlimit(p->J_min - 1, *p), L) : L;
    double2 *d_flm, *d_w, *d_s;
    if (synth) {  // accumulates into flm (src/c/s2let_transform_axisym_lm.c:170-196)
      d_flm = io.inout<double2>(flm, (int64_t)L * L);
      d_w = io.in<double2>(fwav, tot);
      d_s = io.in<double2>(fscal, (int64_t)bs * bs);
    } else {
      d_flm = io.in<double2>(flm, (int64_t)L * L);
      d_w = io.inout<double2>(fwav, tot);
      d_s = io.inout<double2>(fscal, (int64_t)bs * bs);
    }
    const double *d_wl = io.in<double>(wav_lm, (int64_t)(J + 1) * L);
    const double *d_sl = io.in<double>(scal_lm, L);
    const int *d_bl = io.in<int>(bl.data(), (int64_t)bl.size());
    const int64_t *d_off = io.in<int64_t>(off.data(), (int64_t)off.size());
    s2g::axisym_lm(d_flm, d_w, d_s, d_wl, d_sl, d_bl, d_off, p->J_min, (int)bl.size(), L, bs, synth, st);
    io.finish();
  });
}

void threshold_call(const char *fn, double *g, const double *thr, const s2let_parameters_t *p, bool multires) {
  s2g::guarded(fn, [&] {
    S2G_REQUIRE(p != nullptr && g != nullptr && thr != nullptr, s2g::ERR_INVALID, "NULL argument");
    s2let_parameters_t q = *p;
    q.N = 1;
    q.spin = 0;
    s2g::validate(&q, false);
    s2g::ensure_device();
    cudaStream_t st = s2g::host_stream();
    s2g::Scratch S(st);
    s2g::Staged io(S);
    const int L = p->L, J = s2g::j_max(*p);
    std::vector<int64_t> off;
    int64_t tot = 0;
    for (int j = p->J_min; j <= J; ++j) {
      const int64_t b = multires ? std::min(s2g::bandlimit(j, *p), L) : L;
      off.push_back(tot);
      tot += b * (2 * b - 1);
    }
    double *d_g = io.inout<double>(g, tot);
    const double *d_t = io.in<double>(thr, (int64_t)off.size());
    const int64_t *d_off = io.in<int64_t>(off.data(), (int64_t)off.size());
    s2g::hard_threshold(d_g, d_t, d_off, (int)off.size(), tot, st);
    io.finish();
  });
}

}  // namespace

extern "C" {

void s2let_analysis_lm2lmn(cplx *f_wav_lmn, cplx *f_scal_lm, const cplx *flm, const cplx *wav_lm,
                           const double *scal_l, const s2let_parameters_t *p) {
  lm_split(__func__, 0, f_wav_lmn, f_scal_lm, flm, wav_lm, scal_l, p, false);
}
void s2let_analysis_lm2lmn_real(cplx *f_wav_lmn, cplx *f_scal_lm, const cplx *flm, const cplx *wav_lm,
                                const double *scal_l, const s2let_parameters_t *p) {
  lm_split(__func__, 0, f_wav_lmn, f_scal_lm, flm, wav_lm, scal_l, p, true);
}
void s2let_synthesis_adjoint_lm2lmn(cplx *f_wav_lmn, cplx *f_scal_lm, const cplx *flm, const cplx *wav_lm,
                                    const double *scal_l, const s2let_parameters_t *p) {
  lm_split(__func__, 1, f_wav_lmn, f_scal_lm, flm, wav_lm, scal_l, p, false);
}
void s2let_synthesis_adjoint_lm2lmn_real(cplx *f_wav_lmn, cplx *f_scal_lm, const cplx *flm,
                                         const cplx *wav_lm, const double *scal_l,
                                         const s2let_parameters_t *p) {
  lm_split(__func__, 1, f_wav_lmn, f_scal_lm, flm, wav_lm, scal_l, p, true);
}
void s2let_synthesis_lmn2lm(cplx *flm, const cplx *f_wav_lmn, const cplx *f_scal_lm, const cplx *wav_lm,
                            const double *scal_l, const s2let_parameters_t *p) {
  lm_merge(__func__, 0, flm, f_wav_lmn, f_scal_lm, wav_lm, scal_l, p, false);
}
void s2let_synthesis_lmn2lm_real(cplx *flm, const cplx *f_wav_lmn, const cplx *f_scal_lm, const cplx *wav_lm,
                                 const double *scal_l, const s2let_parameters_t *p) {
  lm_merge(__func__, 0, flm, f_wav_lmn, f_scal_lm, wav_lm, scal_l, p, true);
}
void s2let_analysis_adjoint_lmn2lm(cplx *flm, const cplx *f_wav_lmn, const cplx *f_scal_lm,
                                   const cplx *wav_lm, const double *scal_l, const s2let_parameters_t *p) {
  lm_merge(__func__, 1, flm, f_wav_lmn, f_scal_lm, wav_lm, scal_l, p, false);
}
void s2let_analysis_adjoint_lmn2lm_real(cplx *flm, const cplx *f_wav_lmn, const cplx *f_scal_lm,
                                        const cplx *wav_lm, const double *scal_l,
                                        const s2let_parameters_t *p) {
  lm_merge(__func__, 1, flm, f_wav_lmn, f_scal_lm, wav_lm, scal_l, p, true);
}

void s2let_transform_axisym_lm_wav_analysis(cplx *f_wav_lm, cplx *f_scal_lm, const cplx *flm,
                                            const double *wav_lm, const double *scal_lm,
                                            const s2let_parameters_t *p) {
  axisym_lm_call(__func__, false, false, (cplx *)flm, f_wav_lm, f_scal_lm, wav_lm, scal_lm, p);
}
void s2let_transform_axisym_lm_wav_synthesis(cplx *flm, const cplx *f_wav_lm, const cplx *f_scal_lm,
                                             const double *wav_lm, const double *scal_lm,
                                             const s2let_parameters_t *p) {
  axisym_lm_call(__func__, true, false, flm, (cplx *)f_wav_lm, (cplx *)f_scal_lm, wav_lm, scal_lm, p);
}
void s2let_transform_axisym_lm_wav_analysis_multires(cplx *f_wav_lm, cplx *f_scal_lm, const cplx *flm,
                                                     const double *wav_lm, const double *scal_lm,
                                                     const s2let_parameters_t *p) {
  axisym_lm_call(__func__, false, true, (cplx *)flm, f_wav_lm, f_scal_lm, wav_lm, scal_lm, p);
}
void s2let_transform_axisym_lm_wav_synthesis_multires(cplx *flm, const cplx *f_wav_lm, const cplx *f_scal_lm,
                                                      const double *wav_lm, const double *scal_lm,
                                                      const s2let_parameters_t *p) {
  axisym_lm_call(__func__, true, true, flm, (cplx *)f_wav_lm, (cplx *)f_scal_lm, wav_lm, scal_lm, p);
}

void s2let_transform_axisym_wav_hardthreshold_real(double *g_wav, const double *threshold,
                                                   const s2let_parameters_t *p) {
  threshold_call(__func__, g_wav, threshold, p, false);
}
void s2let_transform_axisym_wav_hardthreshold_multires_real(double *g_wav, const double *threshold,
                                                            const s2let_parameters_t *p) {
  threshold_call(__func__, g_wav, threshold, p, true);
}

}  // extern "C"
