// Exchange-correlation functionals at one grid point, FP64, for the device kernels of the SCF
// (cx_scf.cu) and for host code (the same arithmetic compiled by a C++ compiler).
//
//   LDA_PW  src/exchangeCorrelationPotential.m:82-106 (potential), src/evaluateTotalEnergy.m:29-43
//           (energy): Perdew-Wang 1992 correlation with Slater exchange.
//   LDA_PZ  src/evaluateTotalEnergy.m:44-60 (energy); the reference takes the potential from
//           compiled libxc (src/exchangeCorrelationPotential.m:109-130), restated here from the
//           published Perdew-Zunger 1981 parametrisation and its derivative.
//   GGA_PBE src/exchangeCorrelationPotential.m:156-326 (nspin = 1): Perdew, Burke, Ernzerhof,
//           PRL 77, 3865 (1996) with the PW92 correlation above, as f(rho, sigma) = rho e_xc,
//           sigma = |grad rho|^2.  Its two partial derivatives come from forward-mode dual numbers
//           (value, d/drho, d/dsigma) carried through the same expression, so that they are exact
//           to rounding and follow the energy formula by construction.
#pragma once
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __CUDACC__
#define CX_XC_HD __host__ __device__ __forceinline__
#else
#define CX_XC_HD inline
#endif

namespace cx {
namespace xc {

// exchange-correlation codes of the reference's S.xc (src/initialization.m:145-154)
enum { kLdaPw = 0, kLdaPz = 1, kGgaPbe = 2 };

constexpr double kRhoTol = 1e-14;   // S.xc_rhotol (src/initialization.m:143): densities below it are clipped
constexpr int kGradMaxFDn = 8;      // largest half FD order of the gradient stencils

// LDA_PW: the potential v = d(rho e_xc)/d rho and the correlation energy per particle ec at the
// clipped density rc (the exchange energy is -C2 rc^(4/3), C2 = 0.73855876638202).
CX_XC_HD void lda_pw(double rc, double& v, double& ec) {
  const double A = 0.031091, alpha1 = 0.21370, beta1 = 7.5957, beta2 = 3.5876, beta3 = 1.6382, beta4 = 0.49294;
  const double C3 = 0.9847450218427;
  const double rs = cbrt(0.75 / (M_PI * rc));
  const double srs = sqrt(rs);
  const double Q = 2 * A * (beta1 * srs + beta2 * rs + beta3 * rs * srs + beta4 * rs * rs);
  const double lg = log(1 + 1 / Q);
  const double dQ = A * (beta1 / srs + 2 * beta2 + 3 * beta3 * srs + 4 * beta4 * rs);
  v = -C3 * cbrt(rc) + (-2 * A * (1 + alpha1 * rs)) * lg -
      (rs / 3) * (-2 * A * alpha1 * lg - ((-2 * A * (1 + alpha1 * rs)) * dQ) / (Q * Q + Q));
  ec = -2 * A * (1 + alpha1 * rs) * lg;
}

// LDA_PZ: v and erho = rho e_xc at the clipped density rc.  Correlation: rs >= 1 Pade form
// gamma / (1 + beta1 sqrt(rs) + beta2 rs), rs < 1 A ln rs + B + C rs ln rs + D rs; its potential
// ec - (rs / 3) dec/drs.  Exchange: e_x = -C2 rc^(1/3), v_x = -(3 rc / pi)^(1/3).
CX_XC_HD void lda_pz(double rc, double& v, double& erho) {
  const double A = 0.0311, B = -0.048, C = 0.002, D = -0.0116, g = -0.1423, b1 = 1.0529, b2 = 0.3334;
  const double C2 = 0.73855876638202;
  const double rs = cbrt(0.75 / (M_PI * rc));
  double ec, vc;
  if (rs >= 1.0) {
    const double sq = sqrt(rs);
    const double den = 1.0 + b1 * sq + b2 * rs;
    ec = g / den;
    vc = ec * (1.0 + (7.0 / 6.0) * b1 * sq + (4.0 / 3.0) * b2 * rs) / den;
  } else {
    const double lr = log(rs);
    ec = A * lr + B + C * rs * lr + D * rs;
    vc = A * lr + (B - A / 3.0) + (2.0 / 3.0) * C * rs * lr + (2.0 * D - C) / 3.0 * rs;
  }
  const double c1 = cbrt(rc);
  v = -cbrt(3.0 / M_PI) * c1 + vc;
  erho = ec * rc - C2 * rc * c1;
}

// value and first derivatives in (rho, sigma)
struct Dual {
  double v, r, s;
};
CX_XC_HD Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.r + b.r, a.s + b.s}; }
CX_XC_HD Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.r - b.r, a.s - b.s}; }
CX_XC_HD Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.r * b.v + a.v * b.r, a.s * b.v + a.v * b.s}; }
CX_XC_HD Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v, ib = 1.0 / b.v;
  return Dual{q, (a.r - q * b.r) * ib, (a.s - q * b.s) * ib};
}
CX_XC_HD Dual operator+(double a, Dual b) { return Dual{a + b.v, b.r, b.s}; }
CX_XC_HD Dual operator+(Dual a, double b) { return Dual{a.v + b, a.r, a.s}; }
CX_XC_HD Dual operator-(double a, Dual b) { return Dual{a - b.v, -b.r, -b.s}; }
CX_XC_HD Dual operator-(Dual a, double b) { return Dual{a.v - b, a.r, a.s}; }
CX_XC_HD Dual operator*(double a, Dual b) { return Dual{a * b.v, a * b.r, a * b.s}; }
CX_XC_HD Dual operator/(double a, Dual b) {
  const double q = a / b.v, d = -q / b.v;
  return Dual{q, d * b.r, d * b.s};
}
CX_XC_HD Dual dlog(Dual a) { const double d = 1.0 / a.v; return Dual{log(a.v), d * a.r, d * a.s}; }
CX_XC_HD Dual dexp(Dual a) { const double e = exp(a.v); return Dual{e, e * a.r, e * a.s}; }
CX_XC_HD Dual dsqrt(Dual a) { const double q = sqrt(a.v), d = 0.5 / q; return Dual{q, d * a.r, d * a.s}; }
CX_XC_HD Dual dcbrt(Dual a) { const double q = cbrt(a.v), d = q / (3.0 * a.v); return Dual{q, d * a.r, d * a.s}; }

// GGA_PBE: f = rho e_xc, fr = df/drho, fs = df/dsigma at the clipped density rc and sigma.
CX_XC_HD void pbe(double rc, double sigma, double& f, double& fr, double& fs) {
  const double kappa = 0.804, mu = 0.2195149727645171, beta = 0.066725;
  const double gam = (1.0 - 0.69314718055994531) / (M_PI * M_PI);      // (1 - ln 2) / pi^2
  const double A0 = 0.031091, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  const Dual rho{rc, 1.0, 0.0}, sg{sigma, 0.0, 1.0};
  const Dual kf = dcbrt((3.0 * M_PI * M_PI) * rho);
  const Dual ex_lda = (-0.75 * cbrt(3.0 / M_PI)) * dcbrt(rho);
  const Dual rho2 = rho * rho;
  const Dual s2 = sg / (4.0 * (kf * kf) * rho2);
  const Dual Fx = (1.0 + kappa) - kappa / (1.0 + (mu / kappa) * s2);
  const Dual rs = dcbrt(0.75 / (M_PI * rho));
  const Dual srs = dsqrt(rs);
  const Dual ec = (-2.0 * A0) * (1.0 + a1 * rs) *
                  dlog(1.0 + 1.0 / ((2.0 * A0) * (b1 * srs + b2 * rs + b3 * (rs * srs) + b4 * (rs * rs))));
  const Dual ks2 = (4.0 / M_PI) * kf;
  const Dual t2 = sg / (4.0 * ks2 * rho2);
  const Dual Ac = (beta / gam) / (dexp((-1.0 / gam) * ec) - 1.0);
  const Dual At2 = Ac * t2;
  const Dual H = gam * dlog(1.0 + (beta / gam) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  const Dual F = rho * (ex_lda * Fx + ec + H);
  f = F.v;
  fr = F.r;
  fs = F.s;
}

// ---- GGA gradients on the Cyclix grid (Cychel/gradIndicesValues_cychel.m, k = 0)
// Point p = i + Nx (j + Ny k): r = xin + i dx, theta = j dy, z = k dz.  gr/gt/gz[q] = w1[q] / h
// (first-derivative weights, S.w1) per direction.
struct GgaGrid {
  int32_t Nx, Ny, Nz, FDn;
  double xin, dx, dy, dz, twist;
  double gr[kGradMaxFDn + 1], gt[kGradMaxFDn + 1], gz[kGradMaxFDn + 1];
};

template <bool CLIP>
CX_XC_HD double grad_ld(const double* u, size_t idx) {
  const double v = u[idx];
  return CLIP && v < kRhoTol ? kRhoTol : v;
}

// d/dr, d/dtheta, d/dz of u at (i, j, k): radial neighbours outside [0, Nx) are zero (Dirichlet),
// theta and z wrap (periodic, no Bloch phase: the density is a k = 0 field).  With CLIP the field
// is max(u, S.xc_rhotol) inside the grid.
template <bool CLIP>
CX_XC_HD void grad_rtz(const double* u, const GgaGrid& g, int i, int j, int k, double& dr, double& dt, double& dz) {
  const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
  const size_t row = (size_t)Nx * Ny;
  const size_t p = (size_t)i + (size_t)Nx * j + row * k;
  const size_t pj = (size_t)i + row * k;            // (i, 0, k): the theta line through p
  const size_t pk = (size_t)i + (size_t)Nx * j;     // (i, j, 0): the z line through p
  dr = dt = dz = 0.0;
  for (int q = 1; q <= g.FDn; ++q) {
    const double up = i + q < Nx ? grad_ld<CLIP>(u, p + q) : 0.0;
    const double dn = i - q >= 0 ? grad_ld<CLIP>(u, p - q) : 0.0;
    dr += g.gr[q] * (up - dn);
    const int jp = (j + q) % Ny, jm = ((j - q) % Ny + Ny) % Ny;
    dt += g.gt[q] * (grad_ld<CLIP>(u, pj + (size_t)Nx * jp) - grad_ld<CLIP>(u, pj + (size_t)Nx * jm));
    const int kp = (k + q) % Nz, km = ((k - q) % Nz + Nz) % Nz;
    dz += g.gz[q] * (grad_ld<CLIP>(u, pk + row * kp) - grad_ld<CLIP>(u, pk + row * km));
  }
}

// sin and cos of the local angle phi = theta + twist z of point (j, k)
CX_XC_HD void local_angle(const GgaGrid& g, int j, int k, double& sn, double& cs) {
  const double ph = j * g.dy + g.twist * (k * g.dz);
#ifdef __CUDA_ARCH__
  sincos(ph, &sn, &cs);
#else
  sn = sin(ph);
  cs = cos(ph);
#endif
}

// GGA_PBE, first pass at point p: Cartesian gradient of the clipped density, D_x = cos(phi) d_r -
// sin(phi)/r d_theta, D_y = sin(phi) d_r + cos(phi)/r d_theta, D_z = d_z - twist d_theta;
// sigma = |D rho|^2; f = rho e_xc and its partial derivatives.  Writes vxc = df/drho, erho = f
// and q_d = 2 df/dsigma D_d rho (three N-vectors back to back).
CX_XC_HD void gga_pass1_point(const double* rho, const GgaGrid& g, int p, double* vxc, double* erho, double* q) {
  const size_t N = (size_t)g.Nx * g.Ny * g.Nz;
  const int i = p % g.Nx, t = p / g.Nx, j = t % g.Ny, k = t / g.Ny;
  double dr, dt, dz, sn, cs;
  grad_rtz<true>(rho, g, i, j, k, dr, dt, dz);
  local_angle(g, j, k, sn, cs);
  const double r = g.xin + i * g.dx;
  const double gx = cs * dr - sn / r * dt, gy = sn * dr + cs / r * dt, gz = dz - g.twist * dt;
  const double r0 = rho[p];
  const double rc = r0 < kRhoTol ? kRhoTol : r0;
  double f, fr, fs;
  pbe(rc, gx * gx + gy * gy + gz * gz, f, fr, fs);
  vxc[p] = fr;
  erho[p] = f;
  q[p] = 2.0 * fs * gx;
  q[N + p] = 2.0 * fs * gy;
  q[2 * N + p] = 2.0 * fs * gz;
}

// GGA_PBE, second pass at point p: vxc -= D_x q_x + D_y q_y + D_z q_z, the same operators applied
// to the flux (src/exchangeCorrelationPotential.m:360-362).
CX_XC_HD void gga_pass2_point(const double* q, const GgaGrid& g, int p, double* vxc) {
  const size_t N = (size_t)g.Nx * g.Ny * g.Nz;
  const int i = p % g.Nx, t = p / g.Nx, j = t % g.Ny, k = t / g.Ny;
  double ar, at, az, br, bt, bz, cr, ct, cz, sn, cs;
  grad_rtz<false>(q, g, i, j, k, ar, at, az);
  grad_rtz<false>(q + N, g, i, j, k, br, bt, bz);
  grad_rtz<false>(q + 2 * N, g, i, j, k, cr, ct, cz);
  local_angle(g, j, k, sn, cs);
  const double r = g.xin + i * g.dx;
  vxc[p] -= (cs * ar - sn / r * at) + (sn * br + cs / r * bt) + (cz - g.twist * ct);
}

}  // namespace xc
}  // namespace cx
