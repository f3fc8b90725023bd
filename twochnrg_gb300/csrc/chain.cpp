// Wilson-chain coefficients of a non-flat hybridization (host code).
//
// The Lanczos procedure of CNRGchain::SetChainLanczos (NRGchainClass.cpp:
// 234-520): the band [-(1+offset), 1-offset] is cut logarithmically into
// Mmax = ceil(N/2) intervals on each side (CalcFabmEabm, :641-760: interval m
// of the positive side is [D Lambda^-(m+z), D Lambda^-(m+z-1)], the outermost
// one reaching D), each represented by one level at the Gamma-weighted mean
// energy (or, in the Campo-Oliveira scheme, at int Gamma / int Gamma/w) with
// weight int Gamma; the star of levels is tridiagonalized by the Lanczos
// recurrence in the rescaled units of CNRGchain::RHS and ScaleFactor
// (:187-231), the lost orthogonality of the first 2 mmin vectors restored by
// the Chen-Jayaprakash linear solve at every step (:406-460).  Quadrature:
// adaptive 20-point Gauss-Legendre (an interval is split until its value and
// its halves' sum agree to 1e-14 relative), where the reference calls GSL's
// QAG with tolerances 1e-6; for the smooth band shapes here both are exact to
// rounding.  The small dense solves use LU with partial pivoting.
#include <cmath>
#include <vector>

#include "../../include/twochnrg_gb300.h"

namespace {

struct Band {
  int kind;
  std::vector<double> p;
  // HybFunc_Const, HybFunc_Lorentzian, HybFunc_FromFile (HybFuncDefs.cpp:32-260)
  double gamma(double w) const {
    if (kind == NRG_BAND_CONST) return p.size() == 1 ? p[0] : 1.0;
    if (kind == NRG_BAND_LORENTZIAN) {
      if (p.size() < 6) return 1.0;
      const double e2 = p[1], g2 = p[2], sl = p[4];
      double a = std::pow(w - e2, 2.0) + std::pow(g2, 2.0);
      if (a != 0.0) a = sl * sl * g2 / a;
      return a;
    }
    // table of (omega, Gamma) pairs, linear in between, end values outside
    const size_t n = p.size() / 2;
    if (n == 0) return 0.0;
    if (w <= p[0]) return p[1];
    if (w >= p[2 * (n - 1)]) return p[2 * (n - 1) + 1];
    size_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
      const size_t mid = (lo + hi) / 2;
      if (p[2 * mid] > w) hi = mid; else lo = mid;
    }
    const double t = (w - p[2 * lo]) / (p[2 * hi] - p[2 * lo]);
    return p[2 * lo + 1] + t * (p[2 * hi + 1] - p[2 * lo + 1]);
  }
  // HybFuncWithEn: Gamma(w) w, or Gamma(w) / w (-1 at w = 0) for Campo-Oliveira
  double weighted(double w, int disc) const {
    if (disc == 1) return w != 0.0 ? gamma(w) / w : -1.0;
    return w * gamma(w);
  }
};

struct GaussLegendre20 {
  double x[20], w[20];
  GaussLegendre20() {
    const int n = 20;
    const double pi = 3.141592653589793238462643383279502884197169;
    for (int i = 0; i < n / 2; ++i) {
      double z = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 0.0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
          const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1; p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        const double dz = p1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-17) break;
      }
      x[i] = -z; x[n - 1 - i] = z;
      w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
  }
};

template <class F>
double panel(const F& f, double a, double b, const GaussLegendre20& q) {
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  double s = 0.0;
  for (int i = 0; i < 20; ++i) s += q.w[i] * f(c + h * q.x[i]);
  return s * h;
}

template <class F>
double adapt(const F& f, double a, double b, double whole, int depth, const GaussLegendre20& q) {
  const double m = 0.5 * (a + b);
  const double l = panel(f, a, m, q), r = panel(f, m, b, q);
  const double d = std::fabs(l + r - whole);
  if (depth >= 40 || d <= 1e-14 * std::fabs(l + r) || d <= 1e-300) return l + r;
  return adapt(f, a, m, l, depth + 1, q) + adapt(f, m, b, r, depth + 1, q);
}

template <class F>
double integrate(const F& f, double a, double b) {
  static const GaussLegendre20 q;
  if (a == b) return 0.0;
  return adapt(f, a, b, panel(f, a, b, q), 0, q);
}

// A x = b, A row-major n x n; false if singular.
bool solve(int n, std::vector<double> A, std::vector<double>& b) {
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[(size_t)i * n + k]) > std::fabs(A[(size_t)piv * n + k])) piv = i;
    if (A[(size_t)piv * n + k] == 0.0) return false;
    if (piv != k) {
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)k * n + j], A[(size_t)piv * n + j]);
      std::swap(b[k], b[piv]);
    }
    for (int i = k + 1; i < n; ++i) {
      const double l = A[(size_t)i * n + k] / A[(size_t)k * n + k];
      for (int j = k; j < n; ++j) A[(size_t)i * n + j] -= l * A[(size_t)k * n + j];
      b[i] -= l * b[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= A[(size_t)i * n + j] * b[j];
    b[i] = s / A[(size_t)i * n + i];
  }
  return true;
}

}  // namespace

extern "C" {

nrg_status nrg_chain_lanczos(const nrg_band* band, int nsites, double* chi, double* en, double* fsq) {
  if (!band || nsites < 1 || !chi || !en || !(band->lambda > 1.0) || band->nparams < 0 ||
      (band->nparams > 0 && !band->params) || (band->disc_scheme != 0 && band->disc_scheme != 1) ||
      band->kind < NRG_BAND_CONST || band->kind > NRG_BAND_TABLE)
    return NRG_ERR_ARG;
  if (band->kind == NRG_BAND_LORENTZIAN && band->disc_scheme == 1) return NRG_ERR_ARG;  // no Gamma/w form
  Band B{band->kind, std::vector<double>(band->params, band->params + band->nparams)};
  if (B.kind == NRG_BAND_TABLE && (B.p.size() < 4 || B.p.size() % 2)) return NRG_ERR_ARG;
  const double L = band->lambda, z = band->z, off = band->band_offset;
  const int disc = band->disc_scheme, N = nsites;
  const double sqL = std::sqrt(L);
  // CNRGchain::ScaleFactor (NRGchainClass.cpp:187-202)
  auto SF = [&](int n) { return std::pow(L, 0.5 * (double)n + z - 1.0) / (0.5 * (1.0 + (1.0 / L))); };
  // CNRGchain::RHS with scale = true (:209-231)
  auto RHS = [&](int n, double eam, double um, double um1, double e, double chinm1) {
    eam *= SF(n - 1);
    um *= sqL;
    um1 *= sqL;
    return (eam - e) * um - chinm1 * um1;
  };
  const int Mmax = N % 2 == 0 ? N / 2 : (N + 1) / 2;
  // SetHybRef (:570-590); a table whose Gamma(0) vanishes is referred to 1
  // (CNRGCodeHandler::SetChain, NRGcodehandlerClass.cpp:314-322), as any band is
  const double g0 = B.gamma(0.0);
  const double HybRef = std::fabs(g0) < 1e-20 ? 1.0 : g0;
  auto G = [&](double w) { return B.gamma(w); };
  auto GW = [&](double w) { return B.weighted(w, disc); };
  const double F2 = integrate(G, -(1.0 + off), 1.0 - off) / HybRef;  // CalcF2 (:593-640)
  if (fsq) *fsq = F2;
  const double norm0 = F2 * HybRef;
  std::vector<double> F2a, ea, F2b, eb;
  for (int m = 0; m < Mmax; ++m) {  // CalcFabmEabm (:641-760)
    const double dM = (double)m;
    for (int side = 0; side < 2; ++side) {
      double x0, x1;
      if (side == 0) {
        x1 = (1.0 - off) * std::pow(L, -(dM + z - 1.0));
        x0 = (1.0 - off) * std::pow(L, -(dM + z));
        if (m == 0) x1 = 1.0 - off;
      } else {
        x0 = -(1.0 + off) * std::pow(L, -(dM + z - 1.0));
        x1 = -(1.0 + off) * std::pow(L, -(dM + z));
        if (m == 0) x0 = -(1.0 + off);
      }
      const double I = integrate(G, x0, x1), I2 = integrate(GW, x0, x1);
      double e;
      if (disc == 1) e = I2 != 0.0 ? I / I2 : -1.0;
      else e = I != 0.0 ? I2 / I : -1.0;
      (side == 0 ? F2a : F2b).push_back(I);
      (side == 0 ? ea : eb).push_back(e);
    }
  }
  std::vector<std::vector<double>> u(N, std::vector<double>(Mmax, 0.0)), v(N, std::vector<double>(Mmax, 0.0));
  double nrm = 0.0;
  for (int m = 0; m < Mmax; ++m) {
    u[0][m] = std::sqrt(F2a[m] / norm0);
    v[0][m] = std::sqrt(F2b[m] / norm0);
    nrm += u[0][m] * u[0][m] + v[0][m] * v[0][m];
  }
  nrm = std::sqrt(nrm);
  double e0 = 0.0;
  for (int m = 0; m < Mmax; ++m) {
    if (nrm > 0.0) { u[0][m] /= nrm; v[0][m] /= nrm; }
    e0 += u[0][m] * u[0][m] * ea[m] + v[0][m] * v[0][m] * eb[m];
  }
  en[0] = e0 * SF(-1);
  double c0 = 0.0;
  for (int m = 0; m < Mmax; ++m)
    c0 += std::pow(RHS(0, ea[m], u[0][m], 0.0, en[0], 0.0), 2.0) + std::pow(RHS(0, eb[m], v[0][m], 0.0, en[0], 0.0), 2.0);
  chi[0] = std::sqrt(c0);
  for (int n = 1; n < N; ++n) {
    const int mmin = n % 2 == 0 ? n / 2 : (n - 1) / 2;
    double n2 = 0.0;
    for (int m = mmin; m < Mmax; ++m) {
      double a, b;
      if (n == 1) {
        a = RHS(n - 1, ea[m], u[n - 1][m], 0.0, en[n - 1], 0.0) / chi[n - 1];
        b = RHS(n - 1, eb[m], v[n - 1][m], 0.0, en[n - 1], 0.0) / chi[n - 1];
      } else {
        a = RHS(n - 1, ea[m], u[n - 1][m], u[n - 2][m], en[n - 1], chi[n - 2]) / chi[n - 1];
        b = RHS(n - 1, eb[m], v[n - 1][m], v[n - 2][m], en[n - 1], chi[n - 2]) / chi[n - 1];
      }
      u[n][m] = a; v[n][m] = b;
      n2 += a * a + b * b;
    }
    if (mmin > 0) {
      // Chen-Jayaprakash: the first mmin components of u_n and v_n make
      // vector n orthogonal to vectors 0 .. 2 mmin - 1
      const int nv = 2 * mmin;
      std::vector<double> A((size_t)nv * nv), rhs(nv);
      for (int r = 0; r < nv; ++r) {
        for (int c = 0; c < nv; ++c) A[(size_t)r * nv + c] = c < mmin ? u[r][c] : v[r][c - mmin];
        double s = 0.0;
        for (int m = mmin; m < Mmax; ++m) s += u[r][m] * u[n][m] + v[r][m] * v[n][m];
        rhs[r] = -s;
      }
      if (!solve(nv, A, rhs)) return NRG_ERR_NOT_CONVERGED;
      for (int m = 0; m < mmin; ++m) {
        u[n][m] = rhs[m];
        v[n][m] = rhs[m + mmin];
        n2 += u[n][m] * u[n][m] + v[n][m] * v[n][m];
      }
    }
    n2 = std::sqrt(n2);
    double e = 0.0;
    for (int m = 0; m < Mmax; ++m) {
      if (n2 > 0.0) { u[n][m] /= n2; v[n][m] /= n2; }
      e += u[n][m] * u[n][m] * ea[m] + v[n][m] * v[n][m] * eb[m];
    }
    en[n] = e * SF(n - 1);
    double c = 0.0;
    for (int m = 0; m < Mmax; ++m) {
      const double a = RHS(n, ea[m], u[n][m], u[n - 1][m], en[n], chi[n - 1]);
      const double b = RHS(n, eb[m], v[n][m], v[n - 1][m], en[n], chi[n - 1]);
      c += a * a + b * b;
    }
    chi[n] = std::sqrt(c);
  }
  return NRG_OK;
}

}  // extern "C"
