// pbag_eats.cu - the adaptive EATS light curve (method_eats = "adaptive") on
// the GPU, from the layer dynamics and the comoving histories the step left
// on the device.
//
// One work item = one (query, jet side): the principal jet and, with
// counter_jet, the counter jet are separate items (their sum is taken in the
// reference's order at the end), each a nested quadrature run by one warp:
// phi in [0, pi] outside, 1 - cos(theta) inside (integrate_theta_phi,
// eats.h:587-700; phi_integrand :449-586 with find_jet_edge :103-173;
// costheta_integrand :435-448), by CADRE - m9_adapt with the cautious Romberg
// interval rules and a max-heap of intervals on the error (quadratures.h:
// 1613-2113, 657-770) - or by the fixed trapezoid rule (:939-951). The
// integrand (eats.h:175-232) finds the emission time of a direction on the
// item's mu array, interpolates the dynamics log-linearly in radius
// (fluxDensAdaptiveWithComov, blastwave_radiation.h:75-150) and evaluates
// fluxDens (microphysics.h:1185-1217) on the forward- and reverse-shock
// histories.
//
// The integrand and the inner integral are out-of-line functions: one copy of
// their code serves every call site of the quadratures.
//
// GB300 layout. An FP64 warp instruction holds its sub-partition's FP64 unit
// for 64 cycles however many lanes are active, so lanes of one warp must not
// each follow their own adaptive quadrature (divergent paths issue one after
// another). A warp owns one item: every lane runs the quadratures' control
// with the same values (converged; their identical stores to the interval
// workspace coincide), and the points an inner step needs are evaluated by
// the lanes together - the 2 or 4 new points of a CADRE interval, the 2^k
// odd points of its Romberg refinement, every point of a trapezoid sum -
// while the outer (phi) points, each an inner integral, follow in order.
// Sums over a batch are warp reductions (the reference adds point after
// point: the same terms, another rounding order). Every FP64 quantity that
// does not depend on the direction is
// computed once, in parallel, before the quadratures: each item's mu array
// (nr divisions) and, per layer and segment, the logarithms of the ratios of
// neighbouring dynamics values, so that each log-linear interpolation is one
// exp (ya exp(t ln(yb/ya)), t = ln(x/xa) / ln(xb/xa)) instead of a pow and two
// logs; t is formed once per radius and shared by every quantity. The
// intervals of both quadrature levels live in a per-item workspace in global
// memory (nmax + 8 intervals per level); an item whose integration would need
// more stops with PBAG_ERR_NOMEM instead of growing it.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <vector>

#include "pbag.h"
#include "pbag_const.h"
#include "pbag_ctx_view.h"
#include "pbag_device.cuh"

namespace pbag {
namespace {

constexpr int kEatsThreads = 128;  // four items (warps) per CTA
constexpr int kCrewChunk = 32;     // phi points per batch of the crew kernel
constexpr long kMaxEvals = 10000000L;  // eats.h:536-541
// dynamics interpolated log-linearly in radius, in their pbag_eats_q order
__constant__ const int kLogQ[] = {PBAG_EQ_GAMMA,     PBAG_EQ_BETA,         PBAG_EQ_GAMMA_FSH, PBAG_EQ_THICKNESS,
                         PBAG_EQ_M2,        PBAG_EQ_RHO2,         PBAG_EQ_RSH,       PBAG_EQ_ACC_FRAC,
                         PBAG_EQ_THETA,     PBAG_EQ_GAMMA_RSH,    PBAG_EQ_THICKNESS_RS, PBAG_EQ_M3,
                         PBAG_EQ_RHO3,      PBAG_EQ_RRSH,         PBAG_EQ_ACC_FRAC_RS};
constexpr int kNLog = 15;
static_assert(sizeof(kLogQ) == kNLog * sizeof(int), "kNLog counts kLogQ");
enum : int { kLnR = kNLog, kLnT = kNLog + 1, kNLn = kNLog + 2 };  // ln(R ratio), ln(t_burst ratio)

struct Iv9 {  // an interval of CADRE: f[] = fa, fll, fl, flr, fm, frl, fr, frr, fb
  double a, b, I, err;
  double f[9];
  int refinement;
  // inner integral only: points evaluated ahead of their request (kAhead*
  // bits): own quarters in f[2], f[6], own eighths in f[1], f[3], f[5], f[7],
  // the quarter and eighth points of the two halves a split would make, the
  // sum over the next Romberg level's odd points
  int ahead;
  double hq[4], he[8], rs;
};
enum : int { kAheadQ = 1, kAheadE = 2, kAheadHQ = 4, kAheadHE = 8, kAheadR = 16 };

// e^x for the log-linear interpolation within one step of the dynamics grid,
// where |x| = |t ln(y_{i+1}/y_i)| is small: for |x| <= 1/16 the Taylor series
// through x^9 by Horner's rule (the next term is below 2e-19 relative), nine
// FP64 FMAs instead of a full exp; larger |x| (tested on the exponent bits,
// without an FP64 compare) and non-finite x take exp().
__device__ __forceinline__ double exp_step(double x) {
  if ((__double2hiint(x) & 0x7fffffff) > 0x3FB00000) return exp(x);  // |x| > 1/16
  double p = 1.0 / 362880.0;
  p = fma(p, x, 1.0 / 40320.0);
  p = fma(p, x, 1.0 / 5040.0);
  p = fma(p, x, 1.0 / 720.0);
  p = fma(p, x, 1.0 / 120.0);
  p = fma(p, x, 1.0 / 24.0);
  p = fma(p, x, 1.0 / 6.0);
  p = fma(p, x, 0.5);
  p = fma(p, x, 1.0);
  return fma(p, x, 1.0);
}

// The abscissae of CADRE's interval rules, every operation rounded on its own
// (no contraction into FMAs), so that a point evaluated ahead of its request
// has the request's abscissa bit for bit.
__device__ __forceinline__ double lin2(double ca, double a, double cb, double b) {
  return __dadd_rn(__dmul_rn(ca, a), __dmul_rn(cb, b));
}
__device__ __forceinline__ double mid2(double a, double b) { return __dmul_rn(0.5, __dadd_rn(a, b)); }
__device__ __forceinline__ double romberg_h(double a, double b, int nint) {
  return __ddiv_rn(__dsub_rn(b, a), (double)nint);
}
__device__ __forceinline__ double romberg_x(double a, double h, int j) { return __dadd_rn(a, __dmul_rn(h, (double)j)); }
// the four eighth points of [a, b] in the order fll, flr, frl, frr
__device__ __forceinline__ void eighths(double a, double b, double* x) {
  x[0] = lin2(0.875, a, 0.125, b);
  x[1] = lin2(0.625, a, 0.375, b);
  x[2] = lin2(0.375, a, 0.625, b);
  x[3] = lin2(0.125, a, 0.875, b);
}

struct Heap {  // max-heap on err
  Iv9* h;
  int n, cap;
  __device__ bool insert(const Iv9& v) {
    if (n >= cap) return false;
    int c = n++;
    h[c] = v;
    while (c != 0) {
      const int p = (c - 1) / 2;
      if (!(h[p].err < h[c].err)) break;
      const Iv9 t = h[p];
      h[p] = h[c];
      h[c] = t;
      c = p;
    }
    return true;
  }
  __device__ void extract(Iv9* w) {
    *w = h[0];
    h[0] = h[n - 1];
    --n;
    int p = 0;
    for (;;) {
      const int c1 = 2 * p + 1, c2 = c1 + 1;
      if (c1 >= n) break;
      int c = c1;
      double e = h[c1].err;
      if (c2 < n && h[c2].err > e) {
        c = c2;
        e = h[c2].err;
      }
      if (e <= h[p].err) break;
      const Iv9 t = h[p];
      h[p] = h[c];
      h[c] = t;
      p = c;
    }
  }
  __device__ double total_I() const {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += h[i].I;
    return s;
  }
  __device__ double total_err() const {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += h[i].err;
    return s;
  }
};

// findIndex (interpolators.h:13-35)
__device__ int find_index(double x, const double* __restrict__ a, int n) {
  if (x <= a[0]) return 0;
  if (x >= a[n - 1]) return n - 2;
  unsigned lo = 0, hi = (unsigned)n - 1;
  while (hi - lo > 1u) {
    const unsigned m = (hi + lo) >> 1;
    if (a[m] > x)
      hi = m;
    else
      lo = m;
  }
  return (int)lo;
}

__device__ __forceinline__ double beta_from_gamma(double g) { return sqrt((g - 1.) * (g + 1.)) / g; }

// computeIntensity (microphysics.h:11-58)
__device__ double intensity_of(double em, double dtau, int method) {
  if (dtau == 0) return em;
  switch (method) {
    case PBAG_TAU_THICK:
      return dtau > 0 ? em / dtau : 0.;
    case PBAG_TAU_SMOOTH:
      return em * (dtau > 0.0 ? -expm1(-dtau) / dtau : expm1(dtau) / dtau);
    case PBAG_TAU_SHARP:
      return dtau > 1.0 ? em / dtau : dtau < -1.0 ? 0.0 : em;
    default: {
      if (!(dtau > 1.e-3)) return em;
      const double e = exp(-dtau);
      const double u = 1. / 2. + e / dtau - (1 - e) / (dtau * dtau);
      return em * (3. * u / dtau);
    }
  }
}

struct EatsArgs {
  pbag_eats_opts o;
  int nr, F;
  const double* nu;         // [F] photon grid
  const double* dyn;        // [nl][PBAG_EQ_N][nr]
  const double* ln;         // [nl][kNLn][nr]: ln(y[i+1]/y[i]) of the interpolated quantities
  const pbag_eats_layer* layers;
  const int64_t* off;       // history rows of the batch's blastwaves
  const double* j_all;
  const double* a_all;
  const pbag_eats_query* q;
  int nq, sides;
  double* mu;               // [items][nr]
  Iv9* ws;                  // [items][cap_phi + cap_theta]
  int cap_phi, cap_theta;
  double* part;             // [items]
  unsigned long long* first;
  int ahead;                // inner-integral points evaluated ahead (PBAG_EATS_AHEAD=0: on request only)
};

// The EATS object of one work item.
struct Eats {
  const EatsArgs& A;
  const pbag_eats_layer L;
  const double* dyn;
  const double* ln;
  const double* mu;
  int64_t r_fs, r_rs;
  double t_obs, nu_obs, sin_obs, cos_obs;
  bool cj;
  int lane;
  long nevals = 0;
  int code = PBAG_OK;
  Heap inner;
  unsigned long long* evals_sh = nullptr;  // the item's count shared by its warps (crew kernel)

  __device__ const double* qv(int k) const { return dyn + (size_t)k * A.nr; }
  // ya (yb/ya)^t with ln(yb/ya) from the table
  __device__ double seg(int li, int a, double t) const {
    return qv(kLogQ[li])[a] * exp_step(t * ln[(size_t)li * A.nr + a]);
  }

  // fluxDens (microphysics.h:1185-1217) + computeFluxDensity (:799-867) on the
  // history rows r0 + ia, r0 + ib
  __device__ double flux_dens(int64_t r0, int ia, int ib, double freq, double theta, double Gamma, double GammaSh,
                              double mu_, double r, double n_prime, double ne, const double* R, int* rc) const {
    const int F = A.F;
    const double* nu = A.nu;
    if (freq >= nu[F - 1] || freq <= nu[0]) {
      *rc = PBAG_ERR_RANGE;
      return 0.;
    }
    const int ia_nu = find_index(freq, nu, F), ib_nu = ia_nu + 1;
    const double* ja = A.j_all + (size_t)(r0 + ia) * F;
    const double* jb = A.j_all + (size_t)(r0 + ib) * F;
    const double* aa = A.a_all + (size_t)(r0 + ia) * F;
    const double* ab = A.a_all + (size_t)(r0 + ib) * F;
    const double x1 = nu[ia_nu], x2 = nu[ib_nu], y1 = R[ia], y2 = R[ib];
    const double x2x1 = x2 - x1, y2y1 = y2 - y1, x2x = x2 - freq, y2y = y2 - r, yy1 = r - y1, xx1 = freq - x1;
    const double w = 1.0 / (x2x1 * y2y1);
    const double em_prime = w * (ja[ia_nu] * x2x * y2y + ja[ib_nu] * xx1 * y2y + jb[ia_nu] * x2x * yy1 +
                                 jb[ib_nu] * xx1 * yy1);
    const double abs_prime = w * (aa[ia_nu] * x2x * y2y + aa[ib_nu] * xx1 * y2y + ab[ia_nu] * x2x * yy1 +
                                  ab[ib_nu] * xx1 * yy1);
    const double beta = beta_from_gamma(Gamma);
    const double delta_D = Gamma * (1.0 - beta * mu_);
    const double em_lab = em_prime / (delta_D * delta_D);
    const double abs_lab = abs_prime * delta_D;
    const double beta_shock = beta_from_gamma(A.o.flux.shock_vel == PBAG_VEL_SHOCK ? GammaSh : Gamma);
    const double ring = 1. - cos(theta) / L.ncells;
    const double dr = ne * cgs::m_p / (2. * cgs::pi_ * cgs::m_p * r * r * ring * Gamma * n_prime);
    const double dtau = mu_ == beta_shock ? 1.0e100 : abs_lab * dr * (1. - mu_ * beta_shock) / (mu_ - beta_shock);
    const double intensity = intensity_of(em_lab, dtau, A.o.flux.method_tau);
    if (intensity < 0 || !isfinite(intensity)) {
      *rc = PBAG_ERR_NONFINITE;
      return 0.;
    }
    const double ashock = 1.0 - mu_ * beta_shock;
    const double lum = A.o.flux.method_ne == PBAG_NE_USE_NPRIME
                           ? intensity * r * r * (dr / ashock)
                           : intensity * ne / (2. * cgs::pi_ * ring) / Gamma / ashock;
    if (lum < 0 || !isfinite(lum)) {
      *rc = PBAG_ERR_NONFINITE;
      return 0.;
    }
    *rc = PBAG_OK;
    return lum;
  }

  // the integrand (eats.h:175-232) with fluxDensAdaptiveWithComov at this
  // lane's own point (sin_phi = sin(i_phi)); *rc: PBAG_OK or where the
  // reference exits
  __device__ __noinline__ double integrand(double i_cos_theta, double sin_phi, int* rc) const {
    *rc = PBAG_OK;
    const double* R = qv(PBAG_EQ_R);
    const int ie = L.i_end_r;
    if (R[0] == 0.0 && R[ie - 1] == 0.0) return 0.0;
    const double a_theta = 2.0 * asin(sqrt(0.5 * (1.0 - i_cos_theta)));
    const double th = cj ? cgs::pi_ - a_theta : a_theta;  // obsAngle / obsAngleCJ
    const double m = sin_obs * (sin(th) * sin_phi) + cos_obs * cos(th);
    if (m < mu[0] || m > mu[ie - 1]) return 0.;
    const int ia = find_index(m, mu, ie), ib = ia + 1;
    const double* tb = qv(PBAG_EQ_TBURST);
    double t_e = tb[ia] + (tb[ib] - tb[ia]) * (m - mu[ia]) / (mu[ib] - mu[ia]);
    if (mu[0] >= m) t_e = -1;  // check_emission_time (eats.h:24-38)
    if (t_e < 0.0 || !isfinite(t_e)) return 0.;
    // radius at t_e, then every quantity at that radius
    const double r =
        R[ia] * exp_step(log(t_e / tb[ia]) / ln[(size_t)kLnT * A.nr + ia] * ln[(size_t)kLnR * A.nr + ia]);
    if (r <= 0.0 || !isfinite(r)) return 0.0;
    const double t = log(r / R[ia]) / ln[(size_t)kLnR * A.nr + ia];
    const double Gamma = seg(0, ia, t), beta = seg(1, ia, t), theta = seg(8, ia, t);
    const double nuprime = (1.0 + A.o.z) * nu_obs * (Gamma * (1.0 - beta * m));
    double flux = flux_dens(r_fs, ia, ib, nuprime, theta, Gamma, seg(2, ia, t), m, r, seg(5, ia, t) / cgs::m_p,
                            seg(4, ia, t) / cgs::m_p, R, rc);
    if (*rc != PBAG_OK) return 0.;
    const double* th_rs = qv(PBAG_EQ_THICKNESS_RS);
    if (r_rs >= 0 && th_rs[ia] > 0 && th_rs[ib] > 0) {
      const double fr = flux_dens(r_rs, ia, ib, nuprime, theta, Gamma, seg(9, ia, t), m, r, seg(12, ia, t) / cgs::m_p,
                                  seg(11, ia, t) / cgs::m_p, R, rc);
      if (*rc != PBAG_OK) return 0.;
      flux += fr;
    }
    return flux;
  }

  // find_jet_edge (eats.h:103-173)
  __device__ double jet_edge(double ph, double th_con_hi) const {
    const double* thj = qv(PBAG_EQ_THETA);
    const int N = L.i_end_r;
    auto angle = [&](double th) {
      const double x = cj ? cgs::pi_ - th : th;
      return sin_obs * (sin(x) * sin(ph)) + cos_obs * cos(x);
    };
    int ia = find_index(angle(th_con_hi), mu, N);
    if (thj[ia] <= th_con_hi && th_con_hi <= thj[ia + 1]) return th_con_hi;
    double theta_a, theta_b;
    if (th_con_hi < thj[ia]) {
      theta_a = th_con_hi;
      theta_b = 0.5 * cgs::pi_;
    } else {
      theta_a = 0.0;
      theta_b = th_con_hi;
    }
    for (int i = 0; theta_b - theta_a > 1.0e-5 && i < 100; ++i) {
      const double c = 0.5 * (theta_a + theta_b);
      ia = find_index(angle(c), mu, N);
      if (c < thj[ia])
        theta_a = c;
      else
        theta_b = c;
    }
    return theta_a;
  }

  __device__ bool stop() const { return code != PBAG_OK; }

  // ---- the inner integral's points, evaluated by the lanes together
  // (costheta_integrand, eats.h:435-448). A batch stops at its first failing
  // point as the sequential loop would; the evaluation count (the reference's
  // 1e7 limit) grows by the batch.
  __device__ void count_evals(int n) {
    if (evals_sh) {
      unsigned long long tot = 0;
      if (lane == 0) tot = atomicAdd(evals_sh, (unsigned long long)n) + (unsigned long long)n;
      tot = __shfl_sync(0xffffffffu, tot, 0);
      if (tot > (unsigned long long)kMaxEvals && code == PBAG_OK) code = PBAG_ERR_EVALS;
      return;
    }
    nevals += n;
    if (nevals > kMaxEvals && code == PBAG_OK) code = PBAG_ERR_EVALS;
  }
  __device__ void first_failure(int rc) {
    const unsigned bad = __ballot_sync(0xffffffffu, rc != PBAG_OK);
    if (bad) code = __shfl_sync(0xffffffffu, rc, __ffs(bad) - 1);
  }
  // The points of one inner integral: the lanes evaluate them together. A
  // batch needs 2-4 points in most steps of the quadrature, and a warp's FP64
  // instruction costs the same however many lanes are active, so the idle
  // lanes evaluate the points the next steps may request (kAhead): a point's
  // value depends on its abscissa alone, the abscissae are formed the same
  // way, so the results are those of evaluating on request, bit for bit,
  // while the chain of dependent batches shrinks (to about a third on the
  // tested light curves). Only the requested points count as evaluations and
  // can stop the quadrature; a point evaluated ahead that fails is dropped.
  struct Inner {
    static constexpr bool kAhead = true;
    static constexpr bool kMergeSplit = false;  // (the ahead batches cover it)
    Eats& e;
    double sphi;
    __device__ void eval(const double* xs, int n, double* ys) {  // n <= 32
      int rc = PBAG_OK;
      const double y = e.lane < n ? e.integrand(1 - xs[e.lane], sphi, &rc) : 0.;
      e.first_failure(rc);
      e.count_evals(n);
      for (int k = 0; k < n; ++k) ys[k] = __shfl_sync(0xffffffffu, y, k);
    }
    // n requested points xs (lanes [0, n)) and na points ahead xa (lanes
    // [n, n + na), n + na <= 32); returns the lanes of xa that failed
    __device__ unsigned eval_ahead(const double* xs, int n, const double* xa, int na, double* ys, double* ya) {
      int rc = PBAG_OK;
      const int l = e.lane;
      const double x = l < n ? xs[l] : l < n + na ? xa[l - n] : 0.;
      const double y = l < n + na ? e.integrand(1 - x, sphi, &rc) : 0.;
      const unsigned bad = __ballot_sync(0xffffffffu, rc != PBAG_OK);
      const unsigned need = (1u << n) - 1u;
      if (bad & need) e.code = __shfl_sync(0xffffffffu, rc, __ffs(bad & need) - 1);
      if (n > 0) e.count_evals(n);
      for (int k = 0; k < n; ++k) ys[k] = __shfl_sync(0xffffffffu, y, k);
      for (int k = 0; k < na; ++k) ya[k] = __shfl_sync(0xffffffffu, y, n + k);
      return (bad >> n) & ((1u << na) - 1u);
    }
    // sum_odd(a, h, nint) for nint / 2 + nint <= 32, with the next level's sum
    // over its odd points (a + h2 j, h2 = (b - a) / 2 nint) in *next (each sum
    // over the lanes in sum_odd's order); returns whether *next is valid
    __device__ double sum_odd_ahead(double a, double b, double h, int nint, double* next, bool* next_ok) {
      const int l = e.lane, m = nint / 2;
      const double h2 = romberg_h(a, b, 2 * nint);
      int rc = PBAG_OK;
      const double x = l < m ? romberg_x(a, h, 2 * l + 1) : l < m + nint ? romberg_x(a, h2, 2 * (l - m) + 1) : 0.;
      const double y = l < m + nint ? e.integrand(1 - x, sphi, &rc) : 0.;
      const unsigned bad = __ballot_sync(0xffffffffu, rc != PBAG_OK);
      const unsigned need = (1u << m) - 1u;
      if (bad & need) e.code = __shfl_sync(0xffffffffu, rc, __ffs(bad & need) - 1);
      e.count_evals(m);
      *next_ok = ((bad >> m) & ((1u << nint) - 1u)) == 0u;
      double s = l < m ? y : 0.;
      double t = __shfl_sync(0xffffffffu, y, min(l + m, 31));
      t = l < nint ? t : 0.;
      for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        t += __shfl_xor_sync(0xffffffffu, t, o);
      }
      *next = 0. + t;  // as sum_odd accumulates its single chunk
      return e.stop() ? 0. : 0. + s;
    }
    // sum of f(a + h j) over odd j < nint
    __device__ double sum_odd(double a, double h, int nint) {
      double s = 0.;
      for (int base = 1; base < nint; base += 64) {
        const int j = base + 2 * e.lane;
        int rc = PBAG_OK;
        double y = j < nint ? e.integrand(1 - romberg_x(a, h, j), sphi, &rc) : 0.;
        e.first_failure(rc);
        e.count_evals(min(32, (nint - base + 1) / 2));
        if (e.stop()) return 0.;
        for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        s += y;
      }
      return s;
    }
    // trap (quadratures.h:939-951)
    __device__ double trap(double xa, double xb, int N) {
      const double dx = (xb - xa) / N;
      double ends[2];
      const double x2[2] = {xa, xb};
      eval(x2, 2, ends);
      if (e.stop()) return 0.;
      double I = 0.5 * (ends[0] + ends[1]);
      for (int base = 1; base < N; base += 32) {
        const int i = base + e.lane;
        int rc = PBAG_OK;
        double y = i < N ? e.integrand(1 - (xa + i * dx), sphi, &rc) : 0.;
        e.first_failure(rc);
        e.count_evals(min(32, N - base));
        if (e.stop()) return 0.;
        for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        I += y;
      }
      return I * dx;
    }
  };
  struct Outer {  // the points of the phi integral: one inner integral each, in order
    static constexpr bool kAhead = false;
    static constexpr bool kMergeSplit = false;
    Eats& e;
    __device__ void eval(const double* xs, int n, double* ys) {
      for (int k = 0; k < n; ++k) {
        ys[k] = e.phi_integrand(xs[k]);
        if (e.stop()) return;
      }
    }
    __device__ double sum_odd(double a, double h, int nint) {
      double s = 0.;
      for (int j = 1; j < nint; j += 2) {
        s += e.phi_integrand(romberg_x(a, h, j));
        if (e.stop()) return 0.;
      }
      return s;
    }
    __device__ double trap(double xa, double xb, int N) {
      const double dx = (xb - xa) / N;
      const double fa = e.phi_integrand(xa);
      if (e.stop()) return 0.;
      double I = 0.5 * (fa + e.phi_integrand(xb));
      for (int i = 1; i < N; i++) {
        I += e.phi_integrand(xa + i * dx);
        if (e.stop()) return 0.0;
      }
      return I * dx;
    }
  };

  // The points of the phi integral spread over the item's W warps (crew
  // kernel): warp w evaluates points w, w + W, ... of a batch (each one inner
  // integral with its own lanes and its own interval workspace) and leaves
  // value and status in shared memory; after the barrier every warp reads the
  // batch in point order, so all warps hold the same values and sums (the
  // sums in the sequential loop's order) and take the same control path,
  // their own copy of the phi intervals included. A batch's status is its
  // first failing point's.
  struct Crew {
    static constexpr bool kAhead = false;
    // a split's halves request their quarter points one after the other: the
    // crew evaluates all four in one batch (eval_each) and the halves take
    // them as evaluated ahead
    static constexpr bool kMergeSplit = true;
    Eats& e;
    double* ysh;
    int* csh;
    int w, W;
    // every point with its own status; the quadrature's status stays as it was
    __device__ void eval_each(const double* xs, int n, double* ys, int* cs) {
      for (int k = w; k < n; k += W) {
        e.code = PBAG_OK;
        const double y = e.phi_integrand(xs[k]);
        if (e.lane == 0) {
          ysh[k] = y;
          csh[k] = e.code;
        }
      }
      __syncthreads();
      for (int k = 0; k < n; ++k) {
        ys[k] = ysh[k];
        cs[k] = csh[k];
      }
      e.code = PBAG_OK;
      done();
    }
    template <class X>
    __device__ void batch(X xk, int n) {  // n <= kCrewChunk; the caller reads ysh, then calls done()
      for (int k = w; k < n; k += W) {
        e.code = PBAG_OK;
        const double y = e.phi_integrand(xk(k));
        if (e.lane == 0) {
          ysh[k] = y;
          csh[k] = e.code;
        }
      }
      __syncthreads();
      int c = PBAG_OK;
      for (int k = 0; k < n && c == PBAG_OK; ++k) c = csh[k];
      e.code = c;
    }
    __device__ void done() { __syncthreads(); }  // every warp has read the batch
    __device__ void eval(const double* xs, int n, double* ys) {
      batch([&](int k) { return xs[k]; }, n);
      for (int k = 0; k < n; ++k) ys[k] = ysh[k];
      done();
    }
    __device__ double sum_odd(double a, double h, int nint) {
      double s = 0.;
      const int m = nint / 2;  // odd j < nint: j = 2 i + 1
      for (int base = 0; base < m; base += kCrewChunk) {
        const int n = min(kCrewChunk, m - base);
        batch([&](int k) { return romberg_x(a, h, 2 * (base + k) + 1); }, n);
        if (!e.stop())
          for (int k = 0; k < n; ++k) s += ysh[k];
        done();
        if (e.stop()) return 0.;
      }
      return s;
    }
    __device__ double trap(double xa, double xb, int N) {
      const double dx = (xb - xa) / N;
      batch([&](int k) { return k == 0 ? xa : xb; }, 2);
      const double fa = ysh[0], fb = ysh[1];
      done();
      if (e.stop()) return 0.;
      double I = 0.5 * (fa + fb);
      for (int base = 1; base < N; base += kCrewChunk) {
        const int n = min(kCrewChunk, N - base);
        batch([&](int k) { return xa + (base + k) * dx; }, n);
        if (!e.stop())
          for (int k = 0; k < n; ++k) I += ysh[k];
        done();
        if (e.stop()) return 0.0;
      }
      return I * dx;
    }
  };

  // Points of [a, b] that later steps may request: its own eighths (with
  // own), then the quarter points of its halves [a, m], [m, b] (m as a split
  // forms it) and their eighth points.
  __device__ static void ahead_points(double a, double b, bool own, double* x) {
    if (own) {
      eighths(a, b, x);
      x += 4;
    }
    const double m = mid2(a, b);
    x[0] = lin2(0.75, a, 0.25, m);
    x[1] = lin2(0.25, a, 0.75, m);
    x[2] = lin2(0.75, m, 0.25, b);
    x[3] = lin2(0.25, m, 0.75, b);
    eighths(a, m, x + 4);
    eighths(m, b, x + 8);
  }
  // keeps the groups of ahead_points' values whose points all succeeded
  __device__ static void keep_ahead(Iv9* i, bool own, const double* y, unsigned bad) {
    if (own) {
      if (!(bad & 0xFu)) {
        i->f[1] = y[0];
        i->f[3] = y[1];
        i->f[5] = y[2];
        i->f[7] = y[3];
        i->ahead |= kAheadE;
      }
      y += 4;
      bad >>= 4;
    }
    if (!(bad & 0xFu)) {
      for (int k = 0; k < 4; ++k) i->hq[k] = y[k];
      i->ahead |= kAheadHQ;
    }
    if (!(bad & 0xFF0u)) {
      for (int k = 0; k < 8; ++k) i->he[k] = y[4 + k];
      i->ahead |= kAheadHE;
    }
  }

  // CADRE's interval rules (cadreProcessInterval, quadratures.h:1653-1937)
  template <class B>
  __device__ int process(B& fb, Iv9* i) {
    const double scaleTol = 0.2;
    int count = 0;
    if (i->refinement < 4) {
      const double fa = i->f[0], fm = i->f[4], fb_ = i->f[8];
      double fl, fr;
      if (i->refinement == 0) {
        const double xs[2] = {lin2(0.75, i->a, 0.25, i->b), lin2(0.25, i->a, 0.75, i->b)};
        double ys[2];
        if (i->ahead & kAheadQ) {  // evaluated ahead
          ys[0] = i->f[2];
          ys[1] = i->f[6];
          if constexpr (B::kAhead) count_evals(2);  // (the inner integral's points count)
        } else if constexpr (B::kAhead) {
          if (A.ahead) {  // ahead: own eighths, the quarters and eighths of the halves
            double xa[16], ya[16];
            ahead_points(i->a, i->b, true, xa);
            const unsigned bad = fb.eval_ahead(xs, 2, xa, 16, ys, ya);
            keep_ahead(i, true, ya, bad);
          } else {
            fb.eval(xs, 2, ys);
          }
        } else {
          fb.eval(xs, 2, ys);
        }
        count += 2;
        if (stop()) return count;
        fl = ys[0];
        fr = ys[1];
        i->f[2] = fl;
        i->f[6] = fr;
      } else {
        fl = i->f[2];
        fr = i->f[6];
        i->refinement = 0;
      }
      const double h = 0.25 * (i->b - i->a);
      const double T0 = 2 * h * (fa + fb_);
      const double T1 = 0.5 * T0 + 2 * h * fm;
      const double T2 = 0.5 * T1 + h * (fl + fr);
      const double R0 = (T1 - T0) / (T2 - T1);
      if (R0 > 4 - scaleTol && R0 < 4 + scaleTol) {
        double xs[4];
        eighths(i->a, i->b, xs);
        double v[4];
        if constexpr (B::kAhead) {
          if (i->ahead & kAheadE) {  // evaluated ahead
            v[0] = i->f[1];
            v[1] = i->f[3];
            v[2] = i->f[5];
            v[3] = i->f[7];
            count_evals(4);
          } else if (A.ahead) {  // ahead: the quarters and eighths of the halves
            double xa[12], ya[12];
            ahead_points(i->a, i->b, false, xa);
            const unsigned bad = fb.eval_ahead(xs, 4, xa, 12, v, ya);
            keep_ahead(i, false, ya, bad);
          } else {
            fb.eval(xs, 4, v);
          }
        } else {
          fb.eval(xs, 4, v);
        }
        count += 4;
        if (stop()) return count;
        i->f[1] = v[0];
        i->f[3] = v[1];
        i->f[5] = v[2];
        i->f[7] = v[3];
        i->refinement = 1;
        const double T3 = 0.5 * T2 + 0.5 * h * (v[0] + v[1] + v[2] + v[3]);
        const double R1 = (T2 - T1) / (T3 - T2);
        if (R1 > 4 - scaleTol && R1 < 4 + scaleTol) {
          const double R11 = (4 * T1 - T0) / 3.0;
          const double R21 = (4 * T2 - T1) / 3.0;
          const double R22 = (16 * R21 - R11) / 15.0;
          i->f[0] = T3;
          i->f[1] = (4 * T3 - T2) / 3.0;
          i->f[2] = (16 * i->f[1] - R21) / 15.0;
          i->f[3] = (64 * i->f[2] - R22) / 63.0;
          i->I = i->f[3];
          i->err = fabs((i->f[2] - R22) / 63.0);
          i->refinement = 4;
          return count;
        }
        const double errt = (T3 - T2) / 3.0;
        i->err = fabs(errt);
        i->I = T3 + errt;
        return count;
      }
      if (R0 >= 4 + scaleTol || R0 < 2 || R0 != R0) {
        const double e10 = fabs(T1 - T0), e21 = fabs(T2 - T1);
        i->err = e10 > e21 ? e10 : e21;
        i->I = T2;
        return count;
      }
      const double err = -(T2 - T1) * (T2 - T1) / (T2 - 2 * T1 + T0);
      i->err = fabs(err);
      i->I = fabs(T2 + err) < 1.0e-14 * fabs(T2) ? 1.0e-14 * T2 : T2 + err;
      return count;
    }
    // Romberg mode: one more level of the tableau held in f[]
    int nint = 1;
    for (int n = 0; n < i->refinement; n++) nint *= 2;
    const double h = romberg_h(i->a, i->b, nint);
    double sum;
    if constexpr (B::kAhead) {
      if (i->ahead & kAheadR) {  // evaluated ahead at the previous level
        sum = i->rs;
        count_evals(nint / 2);
        i->ahead &= ~kAheadR;
      } else if (A.ahead && nint / 2 + nint <= 32) {
        bool ok = false;
        sum = fb.sum_odd_ahead(i->a, i->b, h, nint, &i->rs, &ok);
        if (ok) i->ahead |= kAheadR;
      } else {
        sum = fb.sum_odd(i->a, h, nint);
      }
    } else {
      sum = fb.sum_odd(i->a, h, nint);
    }
    count += nint / 2;
    if (stop()) return count;
    double Rnm = i->f[0], Rnmp = i->f[1];
    i->f[0] = 0.5 * i->f[0] + h * sum;
    i->f[1] = (4.0 * i->f[0] - Rnm) / 3.0;
    if (i->refinement == 1) {
      i->I = i->f[1];
      i->err = fabs((i->f[0] - Rnm) / 3.0);
      i->refinement += 1;
      return count;
    }
    double pw = 4.0;
    for (int m = 2; m <= 8; ++m) {
      pw *= 4.0;
      Rnm = Rnmp;
      Rnmp = i->f[m];
      i->f[m] = (pw * i->f[m - 1] - Rnm) / (pw - 1.0);
      if (i->refinement == m) {
        i->I = i->f[m];
        i->err = fabs((i->f[m - 1] - Rnm) / (pw - 1.0));
        i->refinement += 1;
        return count;
      }
    }
    i->I = (262144 * i->f[8] - Rnmp) / 262143.0;
    i->err = fabs((i->f[8] - Rnmp) / 262143.0);
    i->refinement += 1;
    return count;
  }

  // m9_adapt (quadratures.h:1969-2101) with atol 0
  template <class B>
  __device__ double cadre(B& fb, double xa, double xb, int nmax, double rtol, Heap& m) {
    m.n = 0;
    Iv9 i{};
    i.a = xa;
    i.b = xb;
    {
      const double xs[3] = {xa, xb, mid2(xa, xb)};  // cadreInitInterval: f(a), f(b), f(m)
      double ys[3];
      bool done = false;
      if constexpr (B::kAhead) {
        if (A.ahead) {  // ahead: the quarters, then as for a quarter step
          double xa2[18], ya[18];
          xa2[0] = lin2(0.75, xa, 0.25, xb);
          xa2[1] = lin2(0.25, xa, 0.75, xb);
          ahead_points(xa, xb, true, xa2 + 2);
          const unsigned bad = fb.eval_ahead(xs, 3, xa2, 18, ys, ya);
          if (!(bad & 3u)) {
            i.f[2] = ya[0];
            i.f[6] = ya[1];
            i.ahead |= kAheadQ;
          }
          keep_ahead(&i, true, ya + 2, bad >> 2);
          done = true;
        }
      }
      if (!done) fb.eval(xs, 3, ys);
      if (stop()) return 0.0;
      i.f[0] = ys[0];
      i.f[8] = ys[1];
      i.f[4] = ys[2];
    }
    int n = 3 + process(fb, &i);
    if (stop()) return 0.0;
    m.insert(i);
    double I = i.I, err = i.err;
    int num_intervals = 1, num_iterations = 0, last_check = 0;
    while (n < nmax && err > rtol * fabs(I)) {
      m.extract(&i);
      if (i.refinement >= 4) {
        const double oldI = i.I, olderr = i.err;
        n += process(fb, &i);
        if (stop()) return 0.0;
        m.insert(i);
        err += i.err - olderr;
        I += i.I - oldI;
      } else {
        Iv9 i1{}, i2{};  // cadreSplitInterval
        const double xm = mid2(i.a, i.b);
        i1.a = i.a;
        i1.b = xm;
        i2.a = xm;
        i2.b = i.b;
        i1.f[0] = i.f[0];
        i1.f[2] = i.f[1];
        i1.f[4] = i.f[2];
        i1.f[6] = i.f[3];
        i1.f[8] = i.f[4];
        i1.refinement = i.refinement;
        i2.f[0] = i.f[4];
        i2.f[2] = i.f[5];
        i2.f[4] = i.f[6];
        i2.f[6] = i.f[7];
        i2.f[8] = i.f[8];
        i2.refinement = i.refinement;
        if constexpr (B::kMergeSplit) {  // both halves' quarter points in one batch
          if (i.refinement == 0) {
            const double xs[4] = {lin2(0.75, i1.a, 0.25, i1.b), lin2(0.25, i1.a, 0.75, i1.b),
                                  lin2(0.75, i2.a, 0.25, i2.b), lin2(0.25, i2.a, 0.75, i2.b)};
            double ys[4];
            int cs[4];
            fb.eval_each(xs, 4, ys, cs);  // a failing point fails again when its half requests it
            if (cs[0] == PBAG_OK && cs[1] == PBAG_OK) {
              i1.f[2] = ys[0];
              i1.f[6] = ys[1];
              i1.ahead |= kAheadQ;
            }
            if (cs[2] == PBAG_OK && cs[3] == PBAG_OK) {
              i2.f[2] = ys[2];
              i2.f[6] = ys[3];
              i2.ahead |= kAheadQ;
            }
          }
        }
        if constexpr (B::kAhead) {  // the halves' points evaluated ahead
          if (i.refinement == 0 && (i.ahead & kAheadHQ)) {  // (otherwise the parent's eighths are their quarters)
            i1.f[2] = i.hq[0];
            i1.f[6] = i.hq[1];
            i2.f[2] = i.hq[2];
            i2.f[6] = i.hq[3];
            i1.ahead |= kAheadQ;
            i2.ahead |= kAheadQ;
          }
          if (A.ahead && i.refinement == 0 && !(i.ahead & kAheadHQ)) {
            // the halves' quarters were not evaluated ahead: one batch for
            // both halves instead of one each - their quarters and eighths,
            // the quarters of each one's halves, the eighths of the first
            // one's halves (all ahead: process() requests them as usual)
            double xa[28], ya[28];
            xa[0] = lin2(0.75, i1.a, 0.25, i1.b);
            xa[1] = lin2(0.25, i1.a, 0.75, i1.b);
            ahead_points(i1.a, i1.b, true, xa + 2);
            xa[18] = lin2(0.75, i2.a, 0.25, i2.b);
            xa[19] = lin2(0.25, i2.a, 0.75, i2.b);
            {
              double t[16];
              ahead_points(i2.a, i2.b, true, t);
              for (int k = 0; k < 8; ++k) xa[20 + k] = t[k];  // its eighths and its halves' quarters
            }
            const unsigned bad = fb.eval_ahead(nullptr, 0, xa, 28, nullptr, ya);
            if (!(bad & 3u)) {
              i1.f[2] = ya[0];
              i1.f[6] = ya[1];
              i1.ahead |= kAheadQ;
            }
            keep_ahead(&i1, true, ya + 2, bad >> 2);
            if (!((bad >> 18) & 3u)) {
              i2.f[2] = ya[18];
              i2.f[6] = ya[19];
              i2.ahead |= kAheadQ;
            }
            keep_ahead(&i2, true, ya + 20, ((bad >> 20) & 0xFFu) | 0xFF00u);  // its halves' eighths: not evaluated
          }
          if (i.ahead & kAheadHE) {
            i1.f[1] = i.he[0];
            i1.f[3] = i.he[1];
            i1.f[5] = i.he[2];
            i1.f[7] = i.he[3];
            i2.f[1] = i.he[4];
            i2.f[3] = i.he[5];
            i2.f[5] = i.he[6];
            i2.f[7] = i.he[7];
            i1.ahead |= kAheadE;
            i2.ahead |= kAheadE;
          }
        }
        n += process(fb, &i1);
        n += process(fb, &i2);
        if (stop()) return 0.0;
        if (!m.insert(i1) || !m.insert(i2)) {
          code = PBAG_ERR_NOMEM;
          return 0.0;
        }
        num_intervals++;
        err += i1.err + i2.err - i.err;
        I += i1.I + i2.I - i.I;
      }
      if (num_iterations == 2 * last_check) {
        err = m.total_err();
        I = m.total_I();
        last_check = num_intervals;
      }
      num_iterations++;
    }
    return m.total_I();
  }

  // phi_integrand (eats.h:449-586): the inner integral over 1 - cos(theta)
  __device__ __noinline__ double phi_integrand(double a_phi) {
    double theta_1 = L.theta_c_h, theta_0 = L.theta_c_l;
    const double th_1 = jet_edge(a_phi, theta_1);
    const double frac = theta_0 / theta_1;
    theta_0 = frac * th_1;
    theta_1 = th_1;
    if (theta_0 > 0.5 * cgs::pi_) theta_0 = 0.5 * cgs::pi_;
    if (theta_1 > 0.5 * cgs::pi_) theta_1 = 0.5 * cgs::pi_;
    const double s0 = sin(0.5 * theta_0), s1 = sin(0.5 * theta_1);
    Inner fin{*this, sin(a_phi)};
    const double result = A.o.method_quad == PBAG_QUAD_TRAP_FIXED
                              ? fin.trap(2.0 * s0 * s0, 2.0 * s1 * s1, A.o.nmax_theta)
                              : cadre(fin, 2.0 * s0 * s0, 2.0 * s1 * s1, A.o.nmax_theta, A.o.rtol_theta, inner);
    if (result != result || result < 0.0) return 0.;
    return result;
  }
};

// each item's mu array (parsPars, eats.h:941-947): one thread per (item, i)
__global__ void k_eats_mu(EatsArgs A, int items) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)items * A.nr) return;
  const int item = (int)(t / A.nr), i = (int)(t % A.nr);
  const pbag_eats_query q = A.q[item / A.sides];
  const double* d = A.dyn + (size_t)q.layer * PBAG_EQ_N * A.nr;
  A.mu[t] = i < A.layers[q.layer].i_end_r
                ? (d[(size_t)PBAG_EQ_TBURST * A.nr + i] - q.t_obs / (1.0 + A.o.z)) / d[(size_t)PBAG_EQ_R * A.nr + i] *
                      cgs::c_light
                : 0.0;
}

// ln(y[i+1] / y[i]) of every interpolated quantity of every layer
__global__ void k_eats_ln(EatsArgs A, double* ln, int nl) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nl * kNLn * A.nr) return;
  const int i = (int)(t % A.nr), k = (int)((t / A.nr) % kNLn), l = (int)(t / ((int64_t)A.nr * kNLn));
  if (i + 1 >= A.nr) {
    ln[t] = 0.0;
    return;
  }
  const int q = k < kNLog ? kLogQ[k] : k == kLnR ? PBAG_EQ_R : PBAG_EQ_TBURST;
  const double* y = A.dyn + ((size_t)l * PBAG_EQ_N + q) * A.nr;
  ln[t] = log(y[i + 1] / y[i]);
}

__global__ void __launch_bounds__(kEatsThreads) k_eats(EatsArgs A, int items) {
  const int item = blockIdx.x * (kEatsThreads / 32) + (threadIdx.x >> 5);  // one item per warp
  if (item >= items) return;
  const int qi = item / A.sides;
  const pbag_eats_query q = A.q[qi];
  const pbag_eats_layer L = A.layers[q.layer];
  Iv9* ws = A.ws + (size_t)item * (A.cap_phi + A.cap_theta);
  Eats e{A, L, A.dyn + (size_t)q.layer * PBAG_EQ_N * A.nr, A.ln + (size_t)q.layer * kNLn * A.nr,
         A.mu + (size_t)item * A.nr, A.off[L.bw_fs], L.bw_rs >= 0 ? A.off[L.bw_rs] : -1,
         q.t_obs, q.nu_obs};
  e.sin_obs = sin(A.o.theta_obs);
  e.cos_obs = cos(A.o.theta_obs);
  e.cj = (item % A.sides) == 1;
  e.lane = threadIdx.x & 31;
  e.inner = Heap{ws + A.cap_phi, 0, A.cap_theta};
  double I = 0.0;
  const double* tb = e.qv(PBAG_EQ_TBURST);
  if (L.i_end_r > 0 && (q.t_obs < tb[0] || q.t_obs > tb[L.i_end_r - 1])) {  // eats.h:822-827
    e.code = PBAG_ERR_RANGE;
  } else {
    Eats::Outer fo{e};
    if (A.o.method_quad == PBAG_QUAD_TRAP_FIXED) {
      I = fo.trap(0.0, cgs::pi_, A.o.nmax_phi);
    } else {
      Heap outer{ws, 0, A.cap_phi};
      I = e.cadre(fo, 0.0, cgs::pi_, A.o.nmax_phi, A.o.rtol_phi, outer);
    }
  }
  const double Fcoeff = 1.e26 / (4 * cgs::pi_ * A.o.d_l * A.o.d_l);  // cgs2mJy (utils.h:40)
  if (e.lane == 0) {
    A.part[item] = 2 * Fcoeff * I;
    if (e.code != PBAG_OK)
      atomicMin(A.first, ((unsigned long long)qi << 8) | (unsigned long long)(-e.code & 0xff));
  }
}

// One item per CTA of W warps: the phi points of each outer step spread over
// the warps (Eats::Crew), each warp with its own interval workspaces. MINB:
// CTAs per SM the registers are budgeted for - 1 for CADRE (255 registers:
// its points evaluated ahead need them, and a light curve's time is its
// slowest items'), 3 for the fixed trapezoid (168: the items are short and
// many, occupancy counts; measured 20 600 against 18 800 points/s with 255,
// CADRE 2 050 against 2 120 with 168).
template <int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) k_eats_crew(EatsArgs A, int items) {
  const int item = blockIdx.x;
  if (item >= items) return;
  const int w = threadIdx.x >> 5;
  __shared__ double ysh[kCrewChunk];
  __shared__ int csh[kCrewChunk];
  __shared__ unsigned long long evals;
  if (threadIdx.x == 0) evals = 0ull;
  __syncthreads();
  const int qi = item / A.sides;
  const pbag_eats_query q = A.q[qi];
  const pbag_eats_layer L = A.layers[q.layer];
  Iv9* ws = A.ws + ((size_t)item * W + w) * (A.cap_phi + A.cap_theta);
  Eats e{A, L, A.dyn + (size_t)q.layer * PBAG_EQ_N * A.nr, A.ln + (size_t)q.layer * kNLn * A.nr,
         A.mu + (size_t)item * A.nr, A.off[L.bw_fs], L.bw_rs >= 0 ? A.off[L.bw_rs] : -1,
         q.t_obs, q.nu_obs};
  e.sin_obs = sin(A.o.theta_obs);
  e.cos_obs = cos(A.o.theta_obs);
  e.cj = (item % A.sides) == 1;
  e.lane = threadIdx.x & 31;
  e.inner = Heap{ws + A.cap_phi, 0, A.cap_theta};
  e.evals_sh = &evals;
  double I = 0.0;
  const double* tb = e.qv(PBAG_EQ_TBURST);
  if (L.i_end_r > 0 && (q.t_obs < tb[0] || q.t_obs > tb[L.i_end_r - 1])) {  // eats.h:822-827
    e.code = PBAG_ERR_RANGE;
  } else {
    Eats::Crew fo{e, ysh, csh, w, W};
    if (A.o.method_quad == PBAG_QUAD_TRAP_FIXED) {
      I = fo.trap(0.0, cgs::pi_, A.o.nmax_phi);
    } else {
      Heap outer{ws, 0, A.cap_phi};
      I = e.cadre(fo, 0.0, cgs::pi_, A.o.nmax_phi, A.o.rtol_phi, outer);
    }
  }
  const double Fcoeff = 1.e26 / (4 * cgs::pi_ * A.o.d_l * A.o.d_l);  // cgs2mJy (utils.h:40)
  if (threadIdx.x == 0) {
    A.part[item] = 2 * Fcoeff * I;
    if (e.code != PBAG_OK)
      atomicMin(A.first, ((unsigned long long)qi << 8) | (unsigned long long)(-e.code & 0xff));
  }
}

// flux = principal jet + counter jet, in evalFluxDensA's order
__global__ void k_eats_sum(const double* __restrict__ part, int nq, int sides, double* __restrict__ flux) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq) return;
  double f = part[(size_t)t * sides];
  if (sides == 2) f += part[(size_t)t * sides + 1];
  flux[t] = f;
}

}  // namespace
}  // namespace pbag

using namespace pbag;

extern "C" int pbag_eats_flux_a(pbag_ctx* ctx, const pbag_eats_opts* opts, int nl, const pbag_eats_layer* h_layers,
                                int nr, const double* d_dyn, int nbw, const int64_t* offsets, const double* d_j_all,
                                const double* d_a_all, int nq, const pbag_eats_query* d_q, double* d_flux,
                                pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || !opts || nl <= 0 || nr < 2 || nbw <= 0 || nq < 0 || !h_layers || !offsets)
    return PBAG_ERR_ARG;
  const pbag_eats_opts& o = *opts;
  if (o.method_quad != PBAG_QUAD_CADRE && o.method_quad != PBAG_QUAD_TRAP_FIXED) return PBAG_ERR_ARG;
  if (o.nmax_theta < 1 || o.nmax_phi < 1 || o.nmax_theta > (1 << 20) || o.nmax_phi > (1 << 20) ||
      !(o.rtol_theta >= 0) || !(o.rtol_phi >= 0) || !(o.d_l > 0))
    return PBAG_ERR_ARG;
  if (o.flux.shock_vel < PBAG_VEL_SAME_AS_BW || o.flux.shock_vel > PBAG_VEL_SHOCK ||
      o.flux.method_ne < PBAG_NE_USE_NPRIME || o.flux.method_ne > PBAG_NE_USE_NE ||
      o.flux.method_tau < PBAG_TAU_APPROX || o.flux.method_tau > PBAG_TAU_SHARP)
    return PBAG_ERR_ARG;
  for (int l = 0; l < nl; ++l) {
    const pbag_eats_layer& L = h_layers[l];
    if (L.i_end_r < 2 || L.i_end_r > nr || L.bw_fs < 0 || L.bw_fs >= nbw || L.bw_rs >= nbw) return PBAG_ERR_ARG;
    for (int b : {L.bw_fs, L.bw_rs})
      if (b >= 0 && offsets[b + 1] - offsets[b] < L.i_end_r) return PBAG_ERR_ARG;
    if (!(L.ncells > 0) || !(L.theta_c_h > 0) || !(L.theta_c_l >= 0)) return PBAG_ERR_ARG;
  }
  if (nq == 0) {
    if (st) st->code = PBAG_OK;
    return PBAG_OK;
  }
  if (!d_dyn || !d_j_all || !d_a_all || !d_q || !d_flux) return PBAG_ERR_ARG;
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  // the queries' layers are checked on the host
  std::vector<pbag_eats_query> hq((size_t)nq);
  if (cudaMemcpy(hq.data(), d_q, (size_t)nq * sizeof(pbag_eats_query), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PBAG_ERR_CUDA;
  for (const pbag_eats_query& q : hq)
    if (q.layer < 0 || q.layer >= nl || !(q.nu_obs > 0) || !(q.t_obs > 0)) return PBAG_ERR_ARG;

  const int sides = o.counter_jet ? 2 : 1;
  const int items = nq * sides;
  EatsArgs A{};
  A.o = o;
  A.nr = nr;
  A.F = v.F;
  A.nu = v.dg.nu;
  A.dyn = d_dyn;
  A.j_all = d_j_all;
  A.a_all = d_a_all;
  A.q = d_q;
  A.nq = nq;
  A.sides = sides;
  A.cap_phi = o.method_quad == PBAG_QUAD_CADRE ? o.nmax_phi + 8 : 0;
  A.cap_theta = o.method_quad == PBAG_QUAD_CADRE ? o.nmax_theta + 8 : 0;
  const size_t n_ln = (size_t)nl * kNLn * nr, n_mu = (size_t)items * nr;
  // warps per item (PBAG_EATS_WARPS = 1 or 4, default 4): the crew kernel
  // spreads each outer step's phi points over four warps
  int crew = 4;
  if (const char* cw = std::getenv("PBAG_EATS_WARPS")) crew = std::atoi(cw) == 1 ? 1 : 4;
  const char* ah = std::getenv("PBAG_EATS_AHEAD");
  A.ahead = (ah && ah[0] == '0') ? 0 : 1;
  const size_t n_ws = (size_t)items * crew * (A.cap_phi + A.cap_theta);
  double *d_ln = nullptr, *d_mu = nullptr, *d_part = nullptr;
  Iv9* d_ws = nullptr;
  pbag_eats_layer* d_layers = nullptr;
  int64_t* d_off = nullptr;
  unsigned long long* d_first = nullptr;
  cudaError_t e = cudaMalloc(&d_ln, n_ln * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&d_mu, n_mu * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&d_part, (size_t)items * sizeof(double));
  if (e == cudaSuccess && n_ws) e = cudaMalloc(&d_ws, n_ws * sizeof(Iv9));
  if (e == cudaSuccess) e = cudaMalloc(&d_layers, (size_t)nl * sizeof(pbag_eats_layer));
  if (e == cudaSuccess) e = cudaMalloc(&d_off, (size_t)(nbw + 1) * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_first, sizeof(unsigned long long));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_layers, h_layers, (size_t)nl * sizeof(pbag_eats_layer), cudaMemcpyHostToDevice, v.stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_off, offsets, (size_t)(nbw + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, v.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_first, 0xff, sizeof(unsigned long long), v.stream);
  A.ln = d_ln;
  A.mu = d_mu;
  A.part = d_part;
  A.ws = d_ws;
  A.layers = d_layers;
  A.off = d_off;
  A.first = d_first;
  if (e == cudaSuccess) {
    k_eats_ln<<<(unsigned)((n_ln + 255) / 256), 256, 0, v.stream>>>(A, d_ln, nl);
    k_eats_mu<<<(unsigned)((n_mu + 255) / 256), 256, 0, v.stream>>>(A, items);
    if (crew == 1)
      k_eats<<<(items + kEatsThreads / 32 - 1) / (kEatsThreads / 32), kEatsThreads, 0, v.stream>>>(A, items);
    else if (o.method_quad == PBAG_QUAD_CADRE)
      k_eats_crew<4, 1><<<items, 128, 0, v.stream>>>(A, items);
    else
      k_eats_crew<4, 3><<<items, 128, 0, v.stream>>>(A, items);
    k_eats_sum<<<(nq + 127) / 128, 128, 0, v.stream>>>(d_part, nq, sides, d_flux);
    e = cudaGetLastError();
  }
  unsigned long long first = ~0ull;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  cudaFree(d_ln);
  cudaFree(d_mu);
  cudaFree(d_part);
  cudaFree(d_ws);
  cudaFree(d_layers);
  cudaFree(d_off);
  cudaFree(d_first);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? PBAG_ERR_NOMEM : PBAG_ERR_CUDA;
  if (first != ~0ull) {
    const int qi = (int)(first >> 8), code = -(int)(first & 0xffull);
    if (st) {
      st->code = code;
      st->bw = hq[(size_t)qi].layer;
      st->step = qi;
    }
    return code;
  }
  if (st) st->code = PBAG_OK;
  return PBAG_OK;
}
