// Host-side construction of the cubic B-spline TableKernel used by the device
// pair loops (product restatement of the reference table build).
//
//  BSplineKernel<Dim<3>> values/gradients   src/Kernel/BSplineKernelInline.hh:28-93
//  NBSplineKernel<Dim<3>>                    src/Kernel/NBSplineKernel.cc:20-118, NBSplineKernelInline.hh:40-99
//  its volume normalisation                  src/Kernel/VolumeIntegrationFunctions.cc, simpsonsIntegration.hh:19-50
//  TableKernel<Dim<3>> constructor           src/Kernel/TableKernel.cc:169-209
//  sumKernelValues (3-D)                     src/Kernel/TableKernel.cc:53-66
//  QuadraticInterpolator::initialize         src/Utilities/QuadraticInterpolator.cc:60-100
//  CubicHermiteInterpolator                  src/Utilities/CubicHermiteInterpolator.cc:95-180
//  bisectRoot                                src/Utilities/bisectRoot.hh:20-74
//
// The reference fits each quadratic interval with Eigen's 3x3 inverse and
// solves the Hermite knot slopes with Eigen's SparseLU; here the inverse is the
// explicit cofactor formula and the tridiagonal system uses the Thomas
// algorithm.  The resulting coefficients agree to rounding.
#include <algorithm>
#include <cmath>
#include <vector>

namespace sph {
namespace table {

namespace {
const double kA = 1.0 / M_PI;   // BSpline 3-D volume normalisation
const double kExtent = 2.0;

double bsW(double eta) {
  if (eta < 1.0) { const double e2 = eta * eta; return kA * 1.0 * (1.0 - 1.5 * e2 + 0.75 * e2 * eta); }
  if (eta < 2.0) { const double d = 2.0 - eta; return kA * 1.0 * 0.25 * (d * d * d); }
  return 0.0;
}
double bsG(double eta) {
  if (eta < 1.0) return -kA * 1.0 * (3.0 - 2.25 * eta) * eta;
  if (eta < 2.0) { const double d = 2.0 - eta; return -kA * 1.0 * 0.75 * (d * d); }
  return 0.0;
}
double bsG2(double eta) {
  if (eta < 1.0) return -kA * 1.0 * (3 - 4.5 * eta);
  if (eta < 2.0) return kA * 1.0 * 1.5 * (2 - eta);
  return 0.0;
}

struct Quad {
  size_t N1 = 0;
  double xstep = 0;
  std::vector<double> c;
  template <class F>
  void fit(double x0, double x1, size_t n, F f) {
    if (n % 2 == 0) ++n;
    const double st = (x1 - x0) / (n - 1u);
    std::vector<double> y(n);
    for (size_t k = 0; k < n; ++k) y[k] = f(x0 + k * st);
    N1 = (n - 1u) / 2u - 1u;
    xstep = (x1 - x0) / (N1 + 1u);
    c.assign(3 * (N1 + 1u), 0.0);
    for (size_t i0 = 0; i0 <= N1; ++i0) {
      const double a0 = x0 + i0 * xstep, a1 = a0 + 0.5 * xstep, a2 = a0 + xstep;
      const double m[3][3] = {{1.0, a0, a0 * a0}, {1.0, a1, a1 * a1}, {1.0, a2, a2 * a2}};
      const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
      const double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
      const double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
      const double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
      const double inv[3][3] = {
          {c00 / det, (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det, (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det},
          {c01 / det, (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det, (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det},
          {c02 / det, (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det, (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det}};
      const double b[3] = {y[2 * i0], y[2 * i0 + 1], y[2 * i0 + 2]};
      for (int r = 0; r < 3; ++r) c[3 * i0 + r] = inv[r][0] * b[0] + inv[r][1] * b[1] + inv[r][2] * b[2];
    }
  }
  double eval(double x) const {
    const size_t i0 = 3u * std::min(N1, size_t(std::max(0.0, x) / xstep));
    return c[i0] + (c[i0 + 1] + c[i0 + 2] * x) * x;
  }
};

struct Hermite {
  size_t N = 0;
  double xmin = 0, xmax = 0, xstep = 0;
  std::vector<double> v;
  template <class F>
  void fit(double x0, double x1, size_t n, F f) {
    const double st = (x1 - x0) / (n - 1u);
    N = n; xmin = x0; xmax = x1;
    v.assign(2 * N, 0.0);
    for (size_t k = 0; k < n; ++k) v[k] = f(x0 + k * st);
    xstep = (x1 - x0) / (N - 1u);
    // slopes: tridiagonal system (4 on the diagonal, -1/2 off, -1 in the end rows)
    std::vector<double> lo(N, 0.0), di(N, 4.0), up(N, 0.0), rhs(N, 0.0);
    up[0] = -1.0; lo[N - 1] = -1.0;
    rhs[0] = 3.0 * (v[1] - v[0]) / xstep;
    rhs[N - 1] = 3.0 * (v[N - 1] - v[N - 2]) / xstep;
    for (size_t k = 1; k + 1 < N; ++k) { lo[k] = -0.5; up[k] = -0.5; rhs[k] = 1.5 * (v[k + 1] - v[k - 1]) / xstep; }
    std::vector<double> cp(N), dp(N);
    cp[0] = up[0] / di[0]; dp[0] = rhs[0] / di[0];
    for (size_t k = 1; k < N; ++k) {
      const double m = di[k] - lo[k] * cp[k - 1];
      cp[k] = up[k] / m;
      dp[k] = (rhs[k] - lo[k] * dp[k - 1]) / m;
    }
    v[2 * N - 1] = dp[N - 1];
    for (size_t k = N - 1; k-- > 0;) v[N + k] = dp[k] - cp[k] * v[N + k + 1];
  }
  void monotonic() {   // Fritsch-Carlson limiting
    std::vector<double> cg(N - 1);
    for (size_t k = 0; k + 1 < N; ++k) cg[k] = (v[k + 1] - v[k]) * (1.0 / xstep);
    auto g = [&](size_t k) -> double& { return v[N + k]; };
    for (size_t k = 1; k + 1 < N; ++k) {
      if (cg[k - 1] * cg[k] <= 0.0) g(k) = 0.0;
      if (cg[k] == 0.0) { g(k) = 0.0; g(k + 1) = 0.0; }
    }
    bool done = false;
    while (!done) {
      done = true;
      for (size_t k = 0; k + 1 < N; ++k) {
        double al = g(k) / cg[k], be = g(k + 1) / cg[k];
        if (al < 0.0) { g(k) = 0.0; al = 0.0; done = false; }
        if (be < 0.0) { g(k + 1) = 0.0; be = 0.0; done = false; }
        const double tau = 3.0 / std::sqrt(al * al + be * be);
        if (tau < 1.0) { g(k) = 0.99 * tau * al * cg[k]; g(k + 1) = 0.99 * tau * be * cg[k]; done = false; }
      }
    }
  }
  double operator()(double x) const {
    if (x < xmin) return v[0] + v[N] * (x - xmin);
    if (x > xmax) return v[N - 1] + v[2 * N - 1] * (x - xmin);
    const size_t i0 = std::min(N - 2u, size_t(std::max(0.0, x - xmin) / xstep));
    const double t = std::max(0.0, std::min(1.0, (x - xmin - i0 * xstep) / xstep));
    const double t2 = t * t, t3 = t * t2;
    return ((2.0 * t3 - 3.0 * t2 + 1.0) * v[i0] + (-2.0 * t3 + 3.0 * t2) * v[i0 + 1] +
            xstep * ((t3 - 2.0 * t2 + t) * v[N + i0] + (t3 - t2) * v[N + i0 + 1]));
  }
};

bool fuzzyZero(double f, double fuzz) { return std::fabs(f) <= fuzz * std::max(1.0, std::fabs(f)); }

template <class F>
double bisect(F f, double xmin, double xmax) {
  const double fmn = f(xmin), fmx = f(xmax);
  if (fuzzyZero(fmn, 1.0e-10)) return xmin;
  if (fuzzyZero(fmx, 1.0e-10)) return xmax;
  double x0, x1;
  if (fmn < 0.0) { x0 = xmin; x1 = xmax; } else { x0 = xmax; x1 = xmin; }
  for (unsigned it = 0; it < 100u; ++it) {
    const double dx = 0.5 * (x1 - x0), r = x0 + dx;
    if (std::fabs(dx) <= 1.0e-15) return r;
    const double fr = f(r);
    if (fuzzyZero(fr, 1.0e-10)) return r;
    if (fr < 0.0) x0 = r; else x1 = r;
  }
  return 0.0;
}

// The centred cardinal B-spline of a given order (Spheral's NBSplineKernel):
// sum_i (-1)^i C(k, i) (eta - i + k/2)_+^e / e!, k = order + 1, with e = order
// for W, order - 1 for dW/deta and order - 2 for the second derivative;
// extent (order + 1) / 2 (integer division); 3-D volume normalisation by
// Simpson's rule over 10,000 bins of 4 pi r^2 W(r).
struct NBSpline {
  int order;
  double A = 1.0, extent;
  static int factorial(int n) {
    if (n < 0) return 2147483647;
    int r = 1;
    for (int i = 1; i < n + 1; ++i) r *= i;
    return r;
  }
  static int binomial(int n, int m) { return factorial(n) / (factorial(n - m) * factorial(m)); }
  double series(double eta, int e) const {
    const int k = order + 1;
    const double halfk = 0.5 * k;
    double r = 0.0;
    for (int i = 0; i <= k; ++i) {
      const double x = eta - i + halfk;
      r += std::pow(-1.0, i) * binomial(k, i) * (x >= 0.0 ? std::pow(x, e) : 0.0);
    }
    return r;
  }
  double term(double eta, int e) const {
    if (eta >= extent) return 0.0;
    return series(eta, e) * (A * 1.0 / factorial(e));
  }
  double W(double eta) const { return term(eta, std::max(0, order)); }
  double G(double eta) const { return term(eta, std::max(-1, order - 1)); }
  double G2(double eta) const { return term(eta, std::max(-2, order - 2)); }
  explicit NBSpline(int o) : order(o), extent((double)((o + 1) / 2)) {
    const int nb = 10000;
    const double dx = (extent - 0.0) / nb;
    double sum = 0.0;
    for (int i = 0; i < nb + 1; ++i) {
      const double r = 0.0 + i * dx;
      const double f = 4.0 * M_PI * r * r * W(r);
      if (i == 0 || i == nb) sum += f;
      else if (i % 2 == 0) sum += 2.0 * f;
      else sum += 4.0 * f;
    }
    sum *= dx / 3.0;
    A = 1.0 / sum;
  }
};

// Wendland kernels, 3-D forms (src/Kernel/WendlandC2KernelInline.hh,
// WendlandC4KernelInline.hh): extent 1, W(1) = 0.
double wc2W(double e) { const double A = 21.0 / (2.0 * M_PI); return A * 1.0 * (std::pow(1.0 - e, 4) * (1.0 + 4.0 * e)) * (e < 1.0 ? 1.0 : 0.0); }
double wc2G(double e) { const double A = 21.0 / (2.0 * M_PI); return A * 1.0 * (20.0 * std::pow(e - 1.0, 3) * e) * (e < 1.0 ? 1.0 : 0.0); }
double wc2G2(double e) { const double A = 21.0 / (2.0 * M_PI); return A * 1.0 * (20.0 * std::pow(e - 1.0, 2) * (4.0 * e - 1.0)) * (e < 1.0 ? 1.0 : 0.0); }
double wc4W(double e) {
  const double A = 495.0 / (32.0 * M_PI);
  return A * 1.0 * (std::pow(1.0 - e, 6) * (1.0 + 6.0 * e + (35.0 / 3.0) * (e * e))) * (e < 1.0 ? 1.0 : 0.0);
}
double wc4G(double e) {
  const double A = 495.0 / (32.0 * M_PI);
  return A * 1.0 * ((56.0 / 3.0) * std::pow(e - 1.0, 5) * e * (5.0 * e + 1.0)) * (e < 1.0 ? 1.0 : 0.0);
}
double wc4G2(double e) {
  const double A = 495.0 / (32.0 * M_PI);
  return A * 1.0 * ((56.0 / 3.0) * std::pow(e - 1.0, 4) * (35.0 * (e * e) - 4.0 * e - 1.0)) * (e < 1.0 ? 1.0 : 0.0);
}

// TableKernel construction from a base kernel (W, dW/deta, d2W/deta2 at
// Hdet = 1 and its extent).
template <class FW, class FG, class FG2>
int buildTable(double extent, FW fw, FG fg, FG2 fg2, int numPoints, double* w, double* g, double* g2, double* nperh,
               double* wsum, double* meta) {
  if (numPoints < 3) return 2;
  const double kExtent = extent;
  Quad qw, qg, qg2;
  qw.fit(0.0, kExtent, (size_t)numPoints, fw);
  qg.fit(0.0, kExtent, (size_t)numPoints, fg);
  qg2.fit(0.0, kExtent, (size_t)numPoints, fg2);
  const double minNperh = std::max(0.25, 1.1 / kExtent);
  double maxNperh = 64.0;
  if (maxNperh <= minNperh) maxNperh = 4.0 * minNperh;
  auto sph = [&](double eta) { return eta < kExtent ? std::fabs(qg.eval(eta)) : 0.0; };
  auto sumKernel = [&](double nPerh) {
    const double deta = 1.0 / nPerh;
    double r = 0.0, e = deta;
    while (e < kExtent) {
      const double q = e / deta;
      r += 4.0 * M_PI * (q * q) * sph(e);
      e += deta;
    }
    return std::pow(r, 1.0 / 3.0);
  };
  Hermite ws, nh;
  ws.fit(minNperh, maxNperh, (size_t)numPoints, sumKernel);
  nh.fit(ws(minNperh), ws(maxNperh), (size_t)numPoints,
         [&](double W) { return bisect([&](double x) { return ws(x) - W; }, minNperh, maxNperh); });
  ws.monotonic();
  nh.monotonic();
  for (size_t k = 0; k < qw.c.size(); ++k) { w[k] = qw.c[k]; g[k] = qg.c[k]; g2[k] = qg2.c[k]; }
  for (size_t k = 0; k < 2 * (size_t)numPoints; ++k) { nperh[k] = nh.v[k]; wsum[k] = ws.v[k]; }
  meta[0] = (double)qw.N1; meta[1] = qw.xstep; meta[2] = (double)numPoints;
  meta[3] = nh.xmin; meta[4] = nh.xmax; meta[5] = ws.xmin; meta[6] = ws.xmax;
  meta[7] = minNperh; meta[8] = maxNperh;
  return 0;
}
}  // namespace

// Returns 0 on success.  Layouts as documented for sphgpu_build_bspline_table.
int buildBSplineTable(int numPoints, double* w, double* g, double* g2, double* nperh, double* wsum, double* meta) {
  return buildTable(kExtent, bsW, bsG, bsG2, numPoints, w, g, g2, nperh, wsum, meta);
}

// kernel 0: BSplineKernel (order ignored); 1: NBSplineKernel(order), order
// 2..9; 2: WendlandC2Kernel; 3: WendlandC4Kernel.  meta[9] receives the
// kernel extent.
int buildKernelTable(int kernel, int order, int numPoints, double* w, double* g, double* g2, double* nperh,
                     double* wsum, double* meta) {
  if (kernel == 0) {
    const int rc = buildBSplineTable(numPoints, w, g, g2, nperh, wsum, meta);
    meta[9] = kExtent;
    return rc;
  }
  if (kernel == 2 || kernel == 3) {
    const int rc = kernel == 2 ? buildTable(1.0, wc2W, wc2G, wc2G2, numPoints, w, g, g2, nperh, wsum, meta)
                               : buildTable(1.0, wc4W, wc4G, wc4G2, numPoints, w, g, g2, nperh, wsum, meta);
    meta[9] = 1.0;
    return rc;
  }
  if (kernel != 1 || order < 2 || order > 9) return 2;
  const NBSpline k(order);
  const int rc = buildTable(
      k.extent, [&](double x) { return k.W(x); }, [&](double x) { return k.G(x); }, [&](double x) { return k.G2(x); },
      numPoints, w, g, g2, nperh, wsum, meta);
  meta[9] = k.extent;
  return rc;
}
double kernelExtent(int kernel, int order) {
  return kernel == 1 ? (double)((order + 1) / 2) : (kernel == 2 || kernel == 3 ? 1.0 : kExtent);
}

}  // namespace table
}  // namespace sph
