// Per-point arithmetic of the nonlocal atomic force (src/atomicForce.m:254-300), for the device
// kernels of cx_force.cu and for host code (the same functions compiled by a C++ compiler).
//
// For every atom column c (kAngMax columns per atom) and Bloch vector k the force needs three
// projector fields on the grid,
//   Ck = sum_img e^{-i k.(R_J - R_img)} chi_img,   R1 = sum_img ROT00 (...),   R2 = sum_img ROT01 (...),
// ROT = RotM1^fac1 RotM2^fac2 the image's wedge / helical rotation, and their Cartesian gradients
//   D_x = M1 R1 + M2 R2,   D_y = -M1 R2 + M2 R1,   D_z = G_z Ck
// with M1, M2 the x / y derivative stencils whose theta-wrapped entries rotate the (R1, R2) pair
// by the wedge angle L2 and carry the Bloch phase (Cychel/div_gradvec_cychel.m) and G_z the z row
// of the Bloch gradient (Cychel/blochGradient_cychel.m).  The force is then
//   F_J -= occfac 2 w_k sum_n occ_n sum_c gamma_c Re[conj(<psi_n|W Ck_c>) (-<psi_n|W D Ck_c>)].
#pragma once
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __CUDACC__
#define CX_F_HD __host__ __device__ __forceinline__
#else
#define CX_F_HD inline
#endif

namespace cx {
namespace force {

constexpr int kCols = 4;          // projector columns per atom (the library's kAngMax)
constexpr int kMaxFDn = 8;

struct Cd {
  double re, im;
};
CX_F_HD Cd cadd(Cd a, Cd b) { return Cd{a.re + b.re, a.im + b.im}; }
CX_F_HD Cd cscale(double s, Cd a) { return Cd{s * a.re, s * a.im}; }
CX_F_HD Cd cmul(Cd a, Cd b) { return Cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// Grid and Bloch data of one block: point p = i + Nx (j + Ny k), r = xin + i dx, phi = j dy + twist k dz.
struct ForceGrid {
  int32_t Nx, Ny, Nz, FDn;
  double xin, dx, dy, dz, twist;
  double cL2, sL2;                // cos / sin of the wedge angle L2
  Cd ph_tl, ph_tr;                // e^{-i k2 L2}, e^{+i k2 L2}: theta neighbours across the left / right wrap
  Cd ph_zl, ph_zr;                // e^{-i k3 L3}, e^{+i k3 L3}
  double w1[kMaxFDn + 1];         // S.w1
};

// Per (atom, image) segment: its atom, e^{-i k.(R_J - R_img)}, and ROT(1,1), ROT(1,2).
struct SegForce {
  Cd ph;
  double rot00, rot01;
  int32_t atom, pad;
};

inline Cd expi(double a) { return Cd{cos(a), sin(a)}; }

// The Bloch phases of a block's wraps: theta neighbours across the left / right wrap carry
// e^{-+i k2 L2}, z neighbours e^{-+i k3 L3} (Cychel/blochGradient_cychel.m).
inline void set_bloch_phases(ForceGrid& g, const double k[3], double L2, double L3) {
  g.ph_tl = expi(-k[1] * L2);
  g.ph_tr = expi(k[1] * L2);
  g.ph_zl = expi(-k[2] * L3);
  g.ph_zr = expi(k[2] * L3);
}

// The segment table of a block: for segment s of atom seg_atom[s] with image coordinates
// seg_coord[3 s ..] and atom position atom_pos[3 J ..], disp = R_J - R_img,
// ph = e^{-i k.disp} and ROT = RotM1^round(disp_2 / L2) RotM2^round(disp_3 / L3), a rotation about z
// by round(disp_2 / L2) L2 + round(disp_3 / L3) twist L3 (src/atomicForce.m:268-273).
inline void segment_table(int nseg, const int32_t* seg_atom, const double* seg_coord, const double* atom_pos, const double k[3],
                          double L2, double L3, double twist, SegForce* out) {
  for (int s = 0; s < nseg; ++s) {
    const int J = seg_atom[s];
    double disp[3], dot = 0.0;
    for (int d = 0; d < 3; ++d) {
      disp[d] = atom_pos[3 * J + d] - seg_coord[3 * s + d];
      dot += k[d] * disp[d];
    }
    const double ang = round(disp[1] / L2) * L2 + round(disp[2] / L3) * twist * L3;
    out[s].ph = expi(-dot);
    out[s].rot00 = cos(ang);
    out[s].rot01 = -sin(ang);
    out[s].atom = J;
    out[s].pad = 0;
  }
}

// The three projector fields at point p from the point's (segment, chi) entries: fields are
// column-major N x C (C = kCols x atoms), written for every column of every atom.
CX_F_HD void force_fields_point(int p, size_t N, int C, const int32_t* row_ptr, const int32_t* ent_seg, const double* ent_chi,
                                const SegForce* seg, Cd* Ck, Cd* R1, Cd* R2) {
  for (int c = 0; c < C; ++c) {
    Ck[p + N * c] = Cd{0.0, 0.0};
    R1[p + N * c] = Cd{0.0, 0.0};
    R2[p + N * c] = Cd{0.0, 0.0};
  }
  for (int e = row_ptr[p]; e < row_ptr[p + 1]; ++e) {
    const SegForce s = seg[ent_seg[e]];
    for (int l = 0; l < kCols; ++l) {
      const double x = ent_chi[(size_t)e * kCols + l];
      const size_t o = p + N * (size_t)(kCols * s.atom + l);
      const Cd v = cscale(x, s.ph);
      Ck[o] = cadd(Ck[o], v);
      R1[o] = cadd(R1[o], cscale(s.rot00, v));
      R2[o] = cadd(R2[o], cscale(s.rot01, v));
    }
  }
}

// W-weighted projector field and its gradient at point p for column c: out holds four column
// blocks of N x C, [W Ck | W D_x | W D_y | W D_z].
CX_F_HD void force_grad_point(int p, size_t N, int C, int c, const ForceGrid& g, const Cd* Ck, const Cd* R1, const Cd* R2,
                              const double* W, Cd* out) {
  const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
  const int i = p % Nx, t = p / Nx, j = t % Ny, k = t / Ny;
  const size_t row = (size_t)Nx * Ny;
  const size_t col0 = N * (size_t)c;
  const Cd* ck = Ck + col0;
  const Cd* r1 = R1 + col0;
  const Cd* r2 = R2 + col0;
  const double r = g.xin + i * g.dx;
  const double ph = j * g.dy + g.twist * (k * g.dz);
#ifdef __CUDA_ARCH__
  double sn, cs;
  sincos(ph, &sn, &cs);
#else
  const double sn = sin(ph), cs = cos(ph);
#endif
  Cd dx{0.0, 0.0}, dy{0.0, 0.0}, dz{0.0, 0.0};
  for (int q = 1; q <= g.FDn; ++q) {
    const double w = g.w1[q];
    for (int sgn = 1; sgn >= -1; sgn -= 2) {
      // radial neighbour (Dirichlet: nothing beyond the walls)
      const int ii = i + sgn * q;
      if (ii >= 0 && ii < Nx) {
        const size_t o = (size_t)ii + (size_t)Nx * j + row * k;
        const double v1 = sgn * w * cs / g.dx, v2 = sgn * w * sn / g.dx;
        dx = cadd(dx, cadd(cscale(v1, r1[o]), cscale(v2, r2[o])));
        dy = cadd(dy, cadd(cscale(-v1, r2[o]), cscale(v2, r1[o])));
      }
      // theta neighbour: wraps with the Bloch phase and, for the x / y pair, the wedge rotation
      {
        int jj = j + sgn * q;
        int tw = 0;
        while (jj < 0) { jj += Ny; tw = -1; }
        while (jj >= Ny) { jj -= Ny; tw = 1; }
        const size_t o = (size_t)i + (size_t)Nx * jj + row * k;
        const double v1 = sgn * w * (-sn / (r * g.dy)), v2 = sgn * w * (cs / (r * g.dy)), v3 = sgn * w * (-g.twist / g.dy);
        if (tw == 0) {
          dx = cadd(dx, cadd(cscale(v1, r1[o]), cscale(v2, r2[o])));
          dy = cadd(dy, cadd(cscale(-v1, r2[o]), cscale(v2, r1[o])));
          dz = cadd(dz, cscale(v3, ck[o]));
        } else {
          const Cd pt = tw < 0 ? g.ph_tl : g.ph_tr;
          const Cd m1 = cscale(v1 * g.cL2 + tw * v2 * g.sL2, pt);
          const Cd m2 = cscale(v2 * g.cL2 - tw * v1 * g.sL2, pt);
          dx = cadd(dx, cadd(cmul(m1, r1[o]), cmul(m2, r2[o])));
          dy = cadd(dy, cadd(cscale(-1.0, cmul(m1, r2[o])), cmul(m2, r1[o])));
          dz = cadd(dz, cmul(cscale(v3, pt), ck[o]));
        }
      }
      // z neighbour: wraps with the Bloch phase
      {
        int kk = k + sgn * q;
        int zw = 0;
        while (kk < 0) { kk += Nz; zw = -1; }
        while (kk >= Nz) { kk -= Nz; zw = 1; }
        const size_t o = (size_t)i + (size_t)Nx * j + row * kk;
        const double v3 = sgn * w / g.dz;
        if (zw == 0) dz = cadd(dz, cscale(v3, ck[o]));
        else dz = cadd(dz, cmul(cscale(v3, zw < 0 ? g.ph_zl : g.ph_zr), ck[o]));
      }
    }
  }
  const double wp = W[p];
  const size_t NC = N * (size_t)C;
  out[col0 + p] = cscale(wp, ck[p]);
  out[NC + col0 + p] = cscale(wp, dx);
  out[2 * NC + col0 + p] = cscale(wp, dy);
  out[3 * NC + col0 + p] = cscale(wp, dz);
}

// One block's contribution to the nonlocal force from P = psi^H [W Ck | W D_x | W D_y | W D_z]
// (Ns x 4C, column-major): F[J + n_atm q] -= scale sum_c gamma_c sum_n occ_n
// Re[conj(P[n, c]) (-P[n, (q + 1) C + c])], scale = occfac 2 w_k; gamma is n_atm x kCols (zero-padded).
inline void force_accumulate(int Ns, int n_atm, const Cd* P, const double* occ, const double* gamma, double scale, double* F) {
  const int C = kCols * n_atm;
  for (int J = 0; J < n_atm; ++J)
    for (int q = 0; q < 3; ++q) {
      double fk = 0.0;
      for (int l = 0; l < kCols; ++l) {
        const int c = kCols * J + l;
        double s = 0.0;
        for (int n = 0; n < Ns; ++n) {
          const Cd a = P[(size_t)n + (size_t)Ns * c], b = P[(size_t)n + (size_t)Ns * ((q + 1) * (size_t)C + c)];
          s += occ[n] * -(a.re * b.re + a.im * b.im);     // Re(conj(a) (-b))
        }
        fk += gamma[kCols * J + l] * s;
      }
      F[J + (size_t)n_atm * q] -= scale * fk;
    }
}

// Cartesian gradient of a real k = 0 field u at point p (S.grad_1..3 * u): radial neighbours
// beyond the walls are zero, theta and z wrap without phase.  Writes D[p], D[N + p], D[2N + p].
CX_F_HD void real_grad_point(int p, const ForceGrid& g, const double* u, double* D) {
  const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
  const size_t N = (size_t)Nx * Ny * Nz;
  const int i = p % Nx, t = p / Nx, j = t % Ny, k = t / Ny;
  const size_t row = (size_t)Nx * Ny;
  double dr = 0.0, dt = 0.0, dzz = 0.0;
  for (int q = 1; q <= g.FDn; ++q) {
    const double w = g.w1[q];
    const double up = i + q < Nx ? u[(size_t)p + q] : 0.0;
    const double dn = i - q >= 0 ? u[(size_t)p - q] : 0.0;
    dr += w * (up - dn);
    const int jp = (j + q) % Ny, jm = ((j - q) % Ny + Ny) % Ny;
    dt += w * (u[(size_t)i + (size_t)Nx * jp + row * k] - u[(size_t)i + (size_t)Nx * jm + row * k]);
    const int kp = (k + q) % Nz, km = ((k - q) % Nz + Nz) % Nz;
    dzz += w * (u[(size_t)i + (size_t)Nx * j + row * kp] - u[(size_t)i + (size_t)Nx * j + row * km]);
  }
  dr /= g.dx;
  dt /= g.dy;
  dzz /= g.dz;
  const double r = g.xin + i * g.dx;
  const double ph = j * g.dy + g.twist * (k * g.dz);
#ifdef __CUDA_ARCH__
  double sn, cs;
  sincos(ph, &sn, &cs);
#else
  const double sn = sin(ph), cs = cos(ph);
#endif
  D[p] = cs * dr - sn / r * dt;
  D[N + p] = sn * dr + cs / r * dt;
  D[2 * N + p] = dzz - g.twist * dt;
}

}  // namespace force
}  // namespace cx
