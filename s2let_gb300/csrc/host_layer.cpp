// Host FP64 layer: tiling kernels (scale-discretised, needlet and spline
// profiles), sizes, allocation helpers and the per-scale layout.  Restates
// src/c/s2let_tiling.c, src/c/s2let_math.c, src/c/s2let_helper.c and
// src/c/s2let_alloc.c of the reference; the expressions that decide band-limits
// and tiling values are evaluated in the same order so results agree bit for bit.
#include "host_layer.h"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "common.h"

namespace s2g {

namespace {

enum Kernel { KERNEL_S2DW = 0, KERNEL_NEEDLET = 1, KERNEL_SPLINE = 2 };
// process-global wavelet family, as the reference's s2let_kernel (src/c/s2let_tiling.c:13-14)
std::atomic<int> g_kernel{KERNEL_S2DW};

inline int lmi(int l, int m) { return l * l + l + m; }

double s2dw_integrand(double k, double B) {
  double t = (k - (1 / B)) * (2.0 * B / (B - 1)) - 1;
  return exp(-2.0 / (1.0 - pow(t, 2.0))) / k;
}
double needlet_integrand(double t) { return exp(-1.0 / (1.0 - pow(t, 2.0))); }

// trapezoid rule over n panels, skipping panels with a non-finite node
// (src/c/s2let_math.c:53-95)
template <class F>
double trapezoid(double a, double b, int n, F f) {
  if (a == b) return 0;
  double h = (b - a) / n, sum = 0;
  for (int i = 0; i < n; i++) {
    double f1 = f(a + i * h), f2 = f(a + (i + 1) * h);
    if (std::isfinite(f1) && std::isfinite(f2)) sum += ((f1 + f2) * h) / 2;
  }
  return sum;
}

double bspline3(double x) {
  if (std::fabs(x) < 1e-16) return 0;
  double a[5];
  for (int k = 0; k < 5; ++k) {
    double y = x + (double)(k - 2);
    a[k] = std::fabs(y * y * y);
  }
  return 1. / 12. * (a[0] - 4. * a[1] + 6. * a[2] - 4. * a[3] + a[4]);
}

// cumulative profiles phi2[l + j L], j = 0..J+1 (src/c/s2let_tiling.c:131-199)
std::vector<double> profiles(const s2let_parameters_t &p) {
  const int L = p.L, J = j_max(p);
  const double B = p.B;
  std::vector<double> phi2((size_t)(J + 2) * L, 0.0);
  const int kind = g_kernel.load();
  if (kind == KERNEL_SPLINE) {
    for (int l = 0; l < L; ++l) phi2[l + (size_t)(J + 1) * L] = 1.0;
    for (int j = 1; j <= J + 1; ++j) {
      double bl = (double)L / (double)pow(B, j - 2);
      double *row = &phi2[(size_t)(J + 1 - j) * L];
      row[0] = 1.0;
      for (int l = 1; l < L; ++l) row[l] = (l > bl) ? 0.0 : 1.5 * bspline3(2.0 * (double)l / bl);
    }
    return phi2;
  }
  const int nq = 300;
  double norm = kind == KERNEL_S2DW
                    ? trapezoid(1.0 / B, 1.0, nq, [B](double k) { return s2dw_integrand(k, B); })
                    : trapezoid(-1.0, 1.0, nq, needlet_integrand);
  for (int j = 0; j <= J + 1; j++)
    for (int l = 0; l < L; l++) {
      double v;
      if (l < pow(B, j - 1))
        v = 1;
      else if (l > pow(B, j))
        v = 0;
      else if (kind == KERNEL_S2DW)
        v = trapezoid((double)l / pow(B, j), 1.0, nq, [B](double k) { return s2dw_integrand(k, B); }) / norm;
      else {
        double u = 1.0 - 2.0 * B / (B - 1.0) * (l * pow(B, -j) - 1.0 / B);
        v = trapezoid(-1.0, u, nq, needlet_integrand) / norm;
      }
      phi2[l + (size_t)j * L] = v;
    }
  return phi2;
}

unsigned long choose(int n, int k) {
  if (k > n / 2) k = n - k;
  unsigned long r = 1;
  for (unsigned long i = 1; i <= (unsigned long)k; ++i) {
    r *= (unsigned long)n - i + 1UL;
    r /= i;
  }
  return r;
}

void axisym_kappa(double *kappa, double *kappa0, const s2let_parameters_t &p) {
  const int L = p.L, J = j_max(p);
  std::vector<double> phi2 = profiles(p);
  for (int l = 0; l < L; l++) kappa0[l] = sqrt(phi2[l + (size_t)p.J_min * L]);
  double carry = 0.0;
  for (int j = p.J_min; j <= J; j++) {
    double *k = kappa + (size_t)j * L;
    for (int l = 0; l < L; l++) {
      double t = sqrt(phi2[l + (size_t)(j + 1) * L] - phi2[l + (size_t)j * L]);
      k[l] = std::isfinite(t) ? t : carry;
      carry = t;
    }
    for (int l = 0; l < L; l++)
      if (!std::isfinite(k[l]) && ((int64_t)j * L + l) > 0) k[l] = kappa[(size_t)j * L + l - 1];
  }
}

void direction_coeffs(cplx *s_elm, const s2let_parameters_t &p) {
  const int L = p.L, N = p.N;
  const cplx nu = (N % 2) ? cplx(1, 0) : cplx(0, 1);
  for (int l = 1; l < L; ++l) {
    int g = ((N + l) % 2) ? std::min(N - 1, l) : std::min(N - 1, l - 1);
    for (int m = -l; m <= l; ++m) {
      cplx v = 0.0;
      if (std::abs(m) < N && ((N + m) % 2))
        v = nu * sqrt(choose(g, (int)((unsigned long)(g - m) / 2UL)) / pow(2, g));
      s_elm[lmi(l, m)] = v;
    }
  }
}

double lowering_norm(int l, int s) {
  double f = 1;
  for (int k = -std::abs(s) + 1; k <= std::abs(s); ++k) f *= l + k;
  return s > 0 ? sqrt(f) : sqrt(1.0 / f);
}

int64_t sum_sq(int64_t k) { return k < 0 ? 0 : k * (k + 1) * (2 * k + 1) / 6; }

}  // namespace

// ---------------------------------------------------------------------------

int j_max(const s2let_parameters_t &p) { return (int)ceil(log(p.L) / log(p.B)); }

int bandlimit(int j, const s2let_parameters_t &p) {
  if (g_kernel.load() == KERNEL_SPLINE) {
    int Jmax = j_max(p);
    if (j == Jmax) return p.L;
    return (int)ceil(p.L / pow(p.B, Jmax - j - 2));
  }
  return (int)ceil(pow(p.B, j + 1));
}

int64_t SO3Shape::flmn_size() const {
  const int64_t L2 = (int64_t)L * L;
  if (reality) return (int64_t)N * L2 - sum_sq(N - 1);
  return (int64_t)(2 * N - 1) * L2 - 2 * sum_sq(N - 1);
}

int64_t SO3Shape::index(int l, int m, int n) const {
  const int64_t L2 = (int64_t)L * L;
  int64_t drop = (n <= 0) ? sum_sq(N - 1) - sum_sq(-n) : sum_sq(N - 1) + sum_sq(n - 1);
  return (int64_t)(n + N - 1) * L2 - drop + (int64_t)l * l - (int64_t)n * n + l + m;
}

int64_t SO3Shape::index_real(int l, int m, int n) const {
  return (int64_t)n * L * L - sum_sq(n - 1) + (int64_t)l * l - (int64_t)n * n + l + m;
}

std::vector<int> Layout::directions(int k) const {
  std::vector<int> out;
  const int Nk = Nj[k];
  if (real)
    for (int n = 1 - Nk % 2; n < Nk; n += 2) out.push_back(n);
  else
    for (int n = -Nk + 1; n < Nk; n += 2) out.push_back(n);
  return out;
}

Layout make_layout(const s2let_parameters_t &p, bool real) {
  Layout g;
  g.L = p.L;
  g.N = p.N;
  g.J = j_max(p);
  g.J_min = p.J_min;
  g.spin = real ? 0 : p.spin;
  g.upsample = p.upsample;
  g.real = real;
  g.bl_scal = p.upsample ? p.L : std::min(bandlimit(p.J_min - 1, p), p.L);
  g.woff.push_back(0);
  g.loff.push_back(0);
  for (int j = p.J_min; j <= g.J; ++j) {
    int bl = p.L, Nj = p.N;
    if (!p.upsample) {
      bl = std::min(bandlimit(j, p), p.L);
      Nj = std::min(p.N, bl);
      Nj += (Nj + p.N) % 2;
    }
    SO3Shape s;
    s.L = bl;
    s.N = Nj;
    s.reality = real ? 1 : p.reality;
    s.n_mode_odd = (p.N % 2) ? 0 : 1;
    s.mwss = p.sampling_scheme == S2LET_SAMPLING_MW_SS ? 1 : 0;
    g.j.push_back(j);
    g.bl.push_back(bl);
    g.Nj.push_back(Nj);
    g.so3.push_back(s);
    g.woff.push_back(g.woff.back() + s.f_size());
    g.loff.push_back(g.loff.back() + s.flmn_size());
  }
  return g;
}

void tiling_wavelet(cplx *psi, double *phi, const s2let_parameters_t &p) {
  const int L = p.L, J = j_max(p), os = p.original_spin;
  std::vector<double> kappa((size_t)(J + 1) * L, 0.0), kappa0(L, 0.0);
  std::vector<cplx> s_elm((size_t)L * L, 0.0);
  axisym_kappa(kappa.data(), kappa0.data(), p);
  direction_coeffs(s_elm.data(), p);
  const int lmin = std::max(std::abs(p.spin), std::abs(os));
  for (int l = lmin; l < L; ++l) {
    phi[l] = sqrt((2 * l + 1) / (4.0 * kPi)) * kappa0[l];
    if (os != 0) phi[l] *= lowering_norm(l, os) * pow(-1, os);
  }
  for (int j = p.J_min; j <= J; ++j)
    for (int l = lmin; l < L; ++l)
      for (int m = -l; m <= l; ++m) {
        cplx v = sqrt((2 * l + 1) / (8.0 * kPi * kPi)) * kappa[(size_t)j * L + l] * s_elm[lmi(l, m)];
        if (os != 0) v *= lowering_norm(l, os) * pow(-1, os);
        psi[(size_t)j * L * L + lmi(l, m)] = v;
      }
}

void axisym_kernels(double *wav_lm, double *scal_lm, const s2let_parameters_t &p) {
  const int L = p.L, J = j_max(p);
  std::vector<double> kappa((size_t)(J + 1) * L, 0.0), kappa0(L, 0.0);
  axisym_kappa(kappa.data(), kappa0.data(), p);
  for (int j = p.J_min; j <= J; j++)
    for (int l = 0; l < L; l++) wav_lm[(size_t)j * L + l] = sqrt((2 * l + 1) / (4.0 * kPi)) * kappa[l + (size_t)j * L];
  for (int l = 0; l < L; l++) scal_lm[l] = sqrt((2 * l + 1) / (4.0 * kPi)) * kappa0[l];
}

void validate(const s2let_parameters_t *p, bool check_sampling) {
  S2G_REQUIRE(p != nullptr, ERR_INVALID, "parameters is NULL");
  S2G_REQUIRE(p->L >= 1, ERR_INVALID, "L must be >= 1");
  S2G_REQUIRE(p->L <= 8192, ERR_INVALID, "L must be <= 8192");
  S2G_REQUIRE(p->N >= 1, ERR_INVALID, "N must be >= 1");
  S2G_REQUIRE(p->B > 1.0, ERR_INVALID, "B must be > 1");
  S2G_REQUIRE(std::abs(p->spin) < p->L, ERR_INVALID, "|spin| must be < L");
  S2G_REQUIRE(p->J_min >= 0 && p->J_min <= j_max(*p), ERR_INVALID, "J_min must lie in [0, J]");
  // src/c/s2let_analysis.c:231-246: MW and MWSS, anything else is an error
  if (check_sampling)
    S2G_REQUIRE(p->sampling_scheme == S2LET_SAMPLING_MW || p->sampling_scheme == S2LET_SAMPLING_MW_SS,
                ERR_UNSUPPORTED, "Sampling scheme not supported.");
}

}  // namespace s2g

// ===========================================================================
// C ABI: tiling, sizes, allocation (host)
// ===========================================================================

using s2g::cplx;

extern "C" {

void s2let_switch_wavtype(int typenum) {
  if (typenum == 2)
    s2g::g_kernel = s2g::KERNEL_NEEDLET;
  else if (typenum == 3)
    s2g::g_kernel = s2g::KERNEL_SPLINE;
  else {
    if (typenum != 1) printf("Kernel number should be 1, 2 or 3. Default is 1.\n");
    s2g::g_kernel = s2g::KERNEL_S2DW;
  }
}

int s2let_bandlimit(int j, const s2let_parameters_t *p) { return s2g::bandlimit(j, *p); }

int s2let_L0(int j, const s2let_parameters_t *p) {
  if (s2g::g_kernel.load() == s2g::KERNEL_SPLINE) return 0;
  return (int)ceil(pow(p->B, j - 1));
}

int s2let_j_max(const s2let_parameters_t *p) { return s2g::j_max(*p); }

void s2let_tiling_axisym_allocate(double **kappa, double **kappa0, const s2let_parameters_t *p) {
  *kappa = (double *)calloc((size_t)(s2g::j_max(*p) + 1) * p->L, sizeof(double));
  *kappa0 = (double *)calloc(p->L, sizeof(double));
}
void s2let_tiling_axisym(double *kappa, double *kappa0, const s2let_parameters_t *p) {
  s2g::axisym_kappa(kappa, kappa0, *p);
}
void s2let_tiling_direction_allocate(cplx **s_elm, const s2let_parameters_t *p) {
  *s_elm = (cplx *)calloc((size_t)p->L * p->L, sizeof(cplx));
}
void s2let_tiling_direction(cplx *s_elm, const s2let_parameters_t *p) { s2g::direction_coeffs(s_elm, *p); }
void s2let_tiling_wavelet_allocate(cplx **psi, double **phi, const s2let_parameters_t *p) {
  *psi = (cplx *)calloc((size_t)(s2g::j_max(*p) + 1) * p->L * p->L, sizeof(cplx));
  *phi = (double *)calloc(p->L, sizeof(double));
}
void s2let_tiling_wavelet(cplx *psi, double *phi, const s2let_parameters_t *p) {
  s2g::tiling_wavelet(psi, phi, *p);
}

double s2let_tiling_axisym_check_identity(double *kappa, double *kappa0, const s2let_parameters_t *p) {
  const int L = p->L, J = s2g::j_max(*p);
  double err = 0;
  for (int l = 0; l < L; l++) {
    double s = pow(kappa0[l], 2.0);
    for (int j = 0; j <= J; j++) s += pow(kappa[l + (size_t)j * L], 2.0);
    err = std::max(err, std::fabs(s - 1.0));
  }
  return err;
}
double s2let_tiling_direction_check_identity(cplx *s_elm, const s2let_parameters_t *p) {
  double err = 0.0;
  for (int l = 1; l < p->L; ++l) {
    double s = 0.0;
    for (int m = -l; m <= l; ++m) s += std::norm(s_elm[l * l + l + m]);
    err = std::max(err, std::fabs(s - 1.0));
  }
  return err;
}
double s2let_tiling_wavelet_check_identity(cplx *psi, double *phi, const s2let_parameters_t *p) {
  const int L = p->L, J = s2g::j_max(*p), s = p->spin;
  std::vector<double> id(L, 0.0);
  double err = 0.0;
  for (int l = std::abs(s); l < L; ++l) id[l] += 4.0 * s2g::kPi / (2 * l + 1) * phi[l] * phi[l];
  for (int j = 0; j <= J; ++j) {
    int ind = s * s;
    for (int l = std::abs(s); l < L; ++l)
      for (int m = -l; m <= l; ++m, ++ind)
        id[l] += 8.0 * s2g::kPi * s2g::kPi / (2 * l + 1) * std::norm(psi[(size_t)j * L * L + ind]);
  }
  for (int l = std::abs(s); l < L; ++l) err = std::max(err, std::fabs(id[l] - 1.0));
  return err;
}

double s2let_math_kappa0_quadtrap_s2dw(double a, double b, int n, double B) {
  return s2g::trapezoid(a, b, n, [B](double k) { return s2g::s2dw_integrand(k, B); });
}
double s2let_math_kappa0_quadtrap_needlet(double a, double b, int n) {
  return s2g::trapezoid(a, b, n, s2g::needlet_integrand);
}
double s2let_math_spline_scalingfct(double x, double y) { return 1.5 * s2g::bspline3(2.0 * x / y); }
unsigned long binomial_coefficient(int n, int k, int exact) {
  (void)exact;
  return s2g::choose(n, k);
}

// sizes (src/c/s2let_helper.c) ----------------------------------------------

int s2let_n_phi(const s2let_parameters_t *p) {
  return p->sampling_scheme == S2LET_SAMPLING_MW_SS ? 2 * p->L : 2 * p->L - 1;
}
int s2let_n_theta(const s2let_parameters_t *p) {
  return p->sampling_scheme == S2LET_SAMPLING_MW_SS ? p->L + 1 : p->L;
}
int s2let_n_px(const s2let_parameters_t *p) { return s2let_n_phi(p) * s2let_n_theta(p); }
int s2let_n_lm(const s2let_parameters_t *p) { return p->L * p->L; }
static int scal_bl(const s2let_parameters_t *p) {
  return p->upsample ? p->L : std::min(s2g::bandlimit(p->J_min - 1, *p), p->L);
}
int s2let_n_lm_scal(const s2let_parameters_t *p) { return scal_bl(p) * scal_bl(p); }
int s2let_n_lmn_wav(const s2let_parameters_t *p) {
  int64_t total = 0;
  for (int j = p->J_min; j <= s2g::j_max(*p); ++j) {
    s2g::SO3Shape s;
    s.L = p->L;
    s.N = p->N;
    s.reality = p->reality;
    if (!p->upsample) {
      s.L = std::min(s2g::bandlimit(j, *p), p->L);
      s.N = std::min(p->N, s.L);  // no parity fix here, as src/c/s2let_helper.c:48-52
    }
    total += s.flmn_size();
  }
  return (int)total;
}
int s2let_n_gamma(const s2let_parameters_t *p) { return 2 * p->N - 1; }
int s2let_n_scal(const s2let_parameters_t *p) {
  s2let_parameters_t q = *p;
  q.L = scal_bl(p);
  return s2let_n_phi(&q) * s2let_n_theta(&q);
}
static int64_t so3_f_size(int L, int N, int mwss) {
  return (int64_t)(2 * N - 1) * (mwss ? 2 * L : 2 * L - 1) * (mwss ? L + 1 : L);
}
int s2let_n_wav(const s2let_parameters_t *p) {
  int64_t total = 0;
  const int mwss = p->sampling_scheme == S2LET_SAMPLING_MW_SS;
  for (int j = p->J_min; j <= s2g::j_max(*p); ++j) {
    int bl = p->upsample ? p->L : std::min(s2g::bandlimit(j, *p), p->L);
    total += so3_f_size(bl, p->N, mwss);  // N, not N_j: src/c/s2let_helper.c:78-95
  }
  return (int)total;
}
int s2let_n_wav_j(int j, const s2let_parameters_t *p) {
  int bl = p->upsample ? p->L : std::min(s2g::bandlimit(j, *p), p->L);
  return (int)so3_f_size(bl, p->N, p->sampling_scheme == S2LET_SAMPLING_MW_SS);
}

// allocation (src/c/s2let_alloc.c) -------------------------------------------

void s2let_allocate_mw(cplx **f, int L) { *f = (cplx *)calloc((size_t)L * (2 * L - 1), sizeof(cplx)); }
void s2let_allocate_mw_real(double **f, int L) { *f = (double *)calloc((size_t)L * (2 * L - 1), sizeof(double)); }
void s2let_allocate_mwss(cplx **f, int L) { *f = (cplx *)calloc((size_t)(2 * L) * (L + 1), sizeof(cplx)); }
void s2let_allocate_mwss_real(double **f, int L) { *f = (double *)calloc((size_t)(2 * L) * (L + 1), sizeof(double)); }
void s2let_allocate_lm(cplx **flm, int L) { *flm = (cplx *)calloc((size_t)L * L, sizeof(cplx)); }
void s2let_allocate_lmn_f_wav(cplx **a, cplx **b, const s2let_parameters_t *p) {
  *a = (cplx *)calloc(s2let_n_lmn_wav(p), sizeof(cplx));
  *b = (cplx *)calloc(s2let_n_lm_scal(p), sizeof(cplx));
}
void s2let_allocate_f_wav(cplx **a, cplx **b, const s2let_parameters_t *p) {
  *a = (cplx *)calloc(s2let_n_wav(p), sizeof(cplx));
  *b = (cplx *)calloc(s2let_n_scal(p), sizeof(cplx));
}
void s2let_allocate_f_wav_real(double **a, double **b, const s2let_parameters_t *p) {
  *a = (double *)calloc(s2let_n_wav(p), sizeof(double));
  *b = (double *)calloc(s2let_n_scal(p), sizeof(double));
}
void s2let_allocate_f_wav_manual(cplx **a, cplx **b, int *wav_bandlimits, int scal_bandlimit, int N,
                                 int J, const s2let_parameters_t *p) {
  (void)N;
  int64_t total = 0;
  for (int j = 0; j <= J; ++j)
    total += so3_f_size(p->upsample ? p->L : wav_bandlimits[j], p->N,
                        p->sampling_scheme == S2LET_SAMPLING_MW_SS);
  s2let_parameters_t q = *p;
  q.L = scal_bandlimit;
  *a = (cplx *)calloc(total, sizeof(cplx));
  *b = (cplx *)calloc((size_t)s2let_n_phi(&q) * s2let_n_theta(&q), sizeof(cplx));
}

void s2let_transform_axisym_lm_allocate_f_wav(cplx **a, cplx **b, const s2let_parameters_t *p) {
  *a = (cplx *)calloc((size_t)(s2g::j_max(*p) + 1 - p->J_min) * p->L * p->L, sizeof(cplx));
  *b = (cplx *)calloc((size_t)p->L * p->L, sizeof(cplx));
}
void s2let_transform_axisym_lm_allocate_f_wav_multires(cplx **a, cplx **b, const s2let_parameters_t *p) {
  int64_t tot = 0;
  for (int j = p->J_min; j <= s2g::j_max(*p); ++j) {
    int64_t bl = std::min(s2g::bandlimit(j, *p), p->L);
    tot += bl * bl;
  }
  int64_t bs = std::min(s2g::bandlimit(p->J_min - 1, *p), p->L);
  *a = (cplx *)calloc(tot, sizeof(cplx));
  *b = (cplx *)calloc(bs * bs, sizeof(cplx));
}
void s2let_transform_axisym_lm_allocate_wav(double **w, double **s, const s2let_parameters_t *p) {
  *w = (double *)calloc((size_t)(s2g::j_max(*p) + 1) * p->L, sizeof(double));
  *s = (double *)calloc(p->L, sizeof(double));
}
void s2let_transform_axisym_lm_wav(double *wav_lm, double *scal_lm, const s2let_parameters_t *p) {
  s2g::axisym_kernels(wav_lm, scal_lm, *p);
}
static int64_t axisym_wav_total(const s2let_parameters_t *p, bool multires, int64_t *scal) {
  const int L = p->L;
  if (!multires) {
    *scal = (int64_t)L * (2 * L - 1);
    return (int64_t)(s2g::j_max(*p) + 1 - p->J_min) * L * (2 * L - 1);
  }
  int64_t tot = 0;
  for (int j = p->J_min; j <= s2g::j_max(*p); ++j) {
    int64_t bl = std::min(s2g::bandlimit(j, *p), L);
    tot += bl * (2 * bl - 1);
  }
  int64_t bs = std::min(s2g::bandlimit(p->J_min - 1, *p), L);
  *scal = bs * (2 * bs - 1);
  return tot;
}
void s2let_transform_axisym_allocate_mw_f_wav(cplx **a, cplx **b, const s2let_parameters_t *p) {
  int64_t sc, t = axisym_wav_total(p, false, &sc);
  *a = (cplx *)calloc(t, sizeof(cplx));
  *b = (cplx *)calloc(sc, sizeof(cplx));
}
void s2let_transform_axisym_allocate_mw_f_wav_multires(cplx **a, cplx **b, const s2let_parameters_t *p) {
  int64_t sc, t = axisym_wav_total(p, true, &sc);
  *a = (cplx *)calloc(t, sizeof(cplx));
  *b = (cplx *)calloc(sc, sizeof(cplx));
}
void s2let_transform_axisym_allocate_mw_f_wav_real(double **a, double **b, const s2let_parameters_t *p) {
  int64_t sc, t = axisym_wav_total(p, false, &sc);
  *a = (double *)calloc(t, sizeof(double));
  *b = (double *)calloc(sc, sizeof(double));
}
void s2let_transform_axisym_allocate_mw_f_wav_multires_real(double **a, double **b,
                                                            const s2let_parameters_t *p) {
  int64_t sc, t = axisym_wav_total(p, true, &sc);
  *a = (double *)calloc(t, sizeof(double));
  *b = (double *)calloc(sc, sizeof(double));
}

double s2let_lm_power(cplx *flm, int L) {
  double t = 0.0;
  for (int i = 0; i < L * L; ++i) t += pow(std::abs(flm[i]), 2.0);
  return t / (L * L);
}

}  // extern "C"

namespace s2g {
int current_kernel_type() { return g_kernel.load(); }
}  // namespace s2g
