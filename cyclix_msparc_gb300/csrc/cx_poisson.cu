// Electrostatic Poisson solve: Alternating Anderson-Richardson (src/aar.m:1-74) on the
// assembled-equivalent operator Lap_std (src/initialization.m:734-740), applied matrix-free:
//   cyclic:  (DL11 + DG1) x + R2inv x DL22^T + x DL33^T,  helical adds x DL22^T and (x DG2^T) DG3^T
// with real coefficients (k = 0) and the boundary conditions of the grid.
// The reference preconditions with ILU(1e-5) (src/initialization.m:752); here the diagonal of
// Lap_std (Jacobi) is used, which keeps every step a streaming pass.  The Anderson least-squares
// step pinv(DF'DF) (DF' res) (aar.m:74) is solved on the device by a one-warp Jacobi
// eigen-decomposition of the m x m normal matrix with MATLAB's pinv tolerance.
//
// The whole iteration runs in one persistent cooperative kernel: its vectors (a few MB, the
// history included) stay in L2, the residual norm and the convergence test are evaluated on the
// device, and the iterations are separated by grid barriers of this file (bounded waits: on a
// timeout the kernel records it in a status word and every block leaves the loop) instead of
// kernel launches and a host round trip per iteration.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cx_common.h"

namespace cx {

constexpr int kAarM = 7;   // Anderson history (poissonSolve.m:36)

__global__ void k_pois_diag(double* dinv, int Nx, int N, double xin, double dx, double d0, double dtheta0, double twist2, int helical) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double r = xin + (double)(i % Nx) * dx;
    const double th = helical ? (twist2 + 1.0 / (r * r)) : 1.0 / (r * r);
    dinv[i] = 1.0 / (d0 + th * dtheta0);
  }
}

// 1/x and 1/sqrt(x) in FP64 from an FP32 estimate and two Newton steps (23 -> 46 -> 92 correct
// bits): a few fused multiply-adds on GB300's narrow FP64 pipe instead of the general division and
// square-root sequences; outside the FP32 range the FP64 operations are used.
__device__ __forceinline__ double rcp64(double x) {
  double y = (double)__frcp_rn((float)x);
  if (!(fabs(y) > 0.0) || !(fabs(y) < 1e37)) return 1.0 / x;
  y = y * fma(-x, y, 2.0);
  y = y * fma(-x, y, 2.0);
  return y;
}
__device__ __forceinline__ double rsqrt64(double x) {
  double y = (double)rsqrtf((float)x);
  if (!(y > 0.0) || !(y < 1e37)) return 1.0 / sqrt(x);
  y = y * fma(-0.5 * x * y, y, 1.5);
  y = y * fma(-0.5 * x * y, y, 1.5);
  return y;
}

// gamma = pinv(A) v for the symmetric kAarM x kAarM A in io (A row-major, then v; gamma written
// after v), MATLAB's pinv tolerance (aar.m:74, mixing.m:104), by one warp.  Jacobi
// eigen-decomposition A = V diag(lambda) V^T in the parallel (round-robin) ordering: the 7
// indices plus a dummy form 4 disjoint pairs per round, 7 rounds per sweep, so the 3 real
// rotations of a round are computed side by side and applied together as A <- J^T A J,
// V <- V J (lane L updates entries L and L + 32 of the 8 x 8 arrays in shared memory).  A pair is
// rotated while a_pq^2 > 1e-30 |a_pp a_qq| (the relative criterion for positive
// semi-definite matrices) and set exactly to zero after its rotation; the sweeps end when a sweep
// rotates nothing (at most 30).  Then gamma = sum over |lambda_k| > 7 max|lambda| eps of
// V_k (V_k . v) / lambda_k.  The whole warp must call it; sA, sV are 64 doubles each, cs 4 x 4.
__device__ __noinline__ void pinv_solve_warp(double* __restrict__ io, double* __restrict__ sA, double* __restrict__ sV,
                                             double* __restrict__ cs) {
  constexpr int M = kAarM, P = 8;
  static_assert(M < P, "one dummy index");
  const int lane = threadIdx.x & 31;
  for (int e = lane; e < P * P; e += 32) {
    const int i = e / P, j = e % P;
    sA[e] = (i < M && j < M) ? io[i * M + j] : 0.0;
    sV[e] = i == j ? 1.0 : 0.0;
  }
  __syncwarp();
  for (int sweep = 0; sweep < 30; ++sweep) {
    bool rotated = false;
    for (int rnd = 0; rnd < P - 1; ++rnd) {
      // pair k of this round: k = 0 is (7, rnd), k = 1..3 are ((rnd + k) % 7, (rnd - k + 7) % 7)
      if (lane < 4) {
        int p = lane == 0 ? P - 1 : (rnd + lane) % (P - 1), q = lane == 0 ? rnd : (rnd - lane + P - 1) % (P - 1);
        if (p > q) { const int t = p; p = q; q = t; }
        double c = 1.0, sn = 0.0, on = 0.0;
        if (q < M) {
          const double app = sA[p * P + p], aqq = sA[q * P + q], apq = sA[p * P + q];
          if (fabs(apq) > 1e-300 && apq * apq > 1e-30 * fabs(app * aqq)) {
            const double th = (aqq - app) * rcp64(2 * apq);
            const double y = th * th + 1;
            const double t = (th >= 0 ? 1.0 : -1.0) * rcp64(fabs(th) + y * rsqrt64(y));
            c = rsqrt64(t * t + 1);
            sn = t * c;
            on = 1.0;
          }
        }
        cs[lane * 4 + 0] = c;
        cs[lane * 4 + 1] = sn;
        cs[lane * 4 + 2] = on;
        cs[lane * 4 + 3] = (double)(p * P + q);
      }
      __syncwarp();
      const bool any = cs[2] + cs[6] + cs[10] + cs[14] > 0;
      if (any) {
        rotated = true;
        // per index i: partner pi, factors (ci, si) with column i of A J = ci col_i + si col_pi
        auto fac = [&](int i, int& pi, double& ci, double& si) {
          pi = i; ci = 1.0; si = 0.0;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int pq = (int)cs[k * 4 + 3], p = pq / P, q = pq % P;
            if (cs[k * 4 + 2] > 0 && (i == p || i == q)) {
              pi = i == p ? q : p;
              ci = cs[k * 4 + 0];
              si = i == p ? -cs[k * 4 + 1] : cs[k * 4 + 1];
            }
          }
        };
        double na[2], nv[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int e = lane + 32 * h, i = e / P, j = e % P;
          int pi, pj;
          double ci, si, cj, sj;
          fac(i, pi, ci, si);
          fac(j, pj, cj, sj);
          na[h] = ci * cj * sA[i * P + j] + ci * sj * sA[i * P + pj] + si * cj * sA[pi * P + j] + si * sj * sA[pi * P + pj];
          if ((pi == j && i != j)) na[h] = 0.0;   // the rotated pair itself
          nv[h] = sV[i * P + j] * cj + sV[i * P + pj] * sj;   // (V J)[i][j]
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          sA[lane + 32 * h] = na[h];
          sV[lane + 32 * h] = nv[h];
        }
      }
      __syncwarp();
    }
    if (!rotated) break;
  }
  if (lane == 0) {
    double nrm = 0;
    for (int i = 0; i < M; ++i) nrm = fmax(nrm, fabs(sA[i * P + i]));
    const double tol = M * nrm * 2.220446049250313e-16;   // MATLAB pinv: max(size(A)) * norm(A) * eps
    double g[M];
    for (int i = 0; i < M; ++i) g[i] = 0;
    for (int k = 0; k < M; ++k) {
      const double lk = sA[k * P + k];
      if (fabs(lk) > tol) {
        double c = 0;
        for (int i = 0; i < M; ++i) c += sV[i * P + k] * io[M * M + i];
        c /= lk;
        for (int i = 0; i < M; ++i) g[i] += sV[i * P + k] * c;
      }
    }
    for (int i = 0; i < M; ++i) io[M * M + M + i] = g[i];
  }
  __syncwarp();
}

__global__ void k_pois_pinv(double* __restrict__ io) {
  __shared__ double sA[64], sV[64], cs[16];
  if (threadIdx.x < 32) pinv_solve_warp(io, sA, sV, cs);
}

// ---------------------------------------------------------------------------- persistent AAR
struct AarArgs {
  int Nx, Ny, Nz, N, F, helical, bcy, bcz;
  double cr2[kMaxFDn + 1], cr1[kMaxFDn + 1], ct2[kMaxFDn + 1], ct1[kMaxFDn + 1], cz2[kMaxFDn + 1], cz1[kMaxFDn + 1];
  const double* f;
  const double* dinv;
  const double* rinv;     // 1 / r per radial node (Nx)
  const double* thsc;     // theta scale per radial node: 1 / r^2, helical tau^2 + 1 / r^2 (Nx)
  double* x0;             // iterate, two buffers (the next iterate is written while the current is read)
  double* x1;
  double* vt;             // helical: D_theta x
  double* res;            // preconditioned residual
  double* xold;
  double* fold;
  double* DX;             // N x m
  double* DF;             // N x m
  double* part;           // per-block partial sums: [2][nblocks] ||r||^2 by iteration parity, then [nblocks][kNormal]
  double* gam;            // Anderson weights (m)
  unsigned* bar;          // barrier arrival word
  int* status;            // 1 when a barrier wait ran out
  double* phi;            // result
  int* out_iters;
  double* out_relres;
  double tol, nb, omega, beta;
  int maxit, p;
};

// Grid barrier of a cooperative launch (every block resident), in the sign-bit form: block 0 adds
// 2^31 - (nblocks - 1) and every other block 1 to one arrival word, so its top bit flips exactly
// when the last block arrives and the word needs no reset.  The wait is bounded (about a second),
// after which *status is set and false is returned to every thread of the block.
__device__ __forceinline__ bool grid_sync(unsigned* bar, int* status) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
    __threadfence();
    const unsigned old = atomicAdd(bar, inc);
    volatile unsigned* w = bar;
    int ok = 1;
    if (((old ^ *w) & 0x80000000u) == 0) {
      const long long t_end = clock64() + (1LL << 31);
      while (((old ^ *w) & 0x80000000u) == 0) {
        if (clock64() > t_end) { ok = 0; atomicExch(status, 1); break; }
        __nanosleep(20);
      }
    }
    __threadfence();
    ok_s = ok && *(volatile int*)status == 0;
  }
  __syncthreads();
  return ok_s != 0;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
  return t;   // valid in thread 0
}
// the normal equations of the Anderson step: upper triangle of DF'DF, then DF'res
constexpr int kNormal = kAarM * (kAarM + 1) / 2 + kAarM;

// block sums of the kNormal values of every thread, written to out[0 .. kNormal) (global);
// red: shared scratch of (blockDim.x / 32) x kNormal doubles
__device__ __forceinline__ void block_sum_many(double (&v)[kNormal], double* red, double* out) {
  static_assert(kNormal >= 32, "one transposed sum per lane");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // values 32 .. kNormal-1: shuffle trees (every lane ends with the warp sum)
#pragma unroll
  for (int k = 32; k < kNormal; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane == 0) red[w * kNormal + k] = v[k];
  }
  // values 0 .. 31: a transposing butterfly (31 shuffles and adds instead of 5 per value, which
  // matters on GB300's narrow FP64 pipe); lane l ends with the warp sum of value l
#pragma unroll
  for (int o = 16, c = 32; o > 0; o >>= 1, c >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < c / 2; ++i) {
      const double keep = up ? v[i + c / 2] : v[i];
      const double send = up ? v[i] : v[i + c / 2];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  red[w * kNormal + lane] = v[0];
  __syncthreads();
  for (int k = threadIdx.x; k < kNormal; k += blockDim.x) {
    double t = 0;
    for (int i = 0; i < nw; ++i) t += red[i * kNormal + k];
    out[k] = t;
  }
  __syncthreads();
}

// sum of the n per-block partials at a (written by other blocks): every thread gets it
__device__ __forceinline__ double sum_partials(const double* a, int n, double* sh) {
  __shared__ double tot;
  if (threadIdx.x < 32) {
    double v = 0;
    for (int i = threadIdx.x; i < n; i += 32) v += __ldcg(a + i);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) tot = v;
  }
  __syncthreads();
  const double t = tot;
  __syncthreads();
  return t;
}

// neighbour in theta / z with the grid's boundary conditions (k = 0: no phase); -1 when zero
__device__ __forceinline__ int wrap_idx(int i, int n, int bc) {
  if (i < 0) return bc ? -1 : i + n;
  if (i >= n) return bc ? -1 : i - n;
  return i;
}
// values of x visible across blocks: load through L2 (the L1 of another SM may hold a stale line)
__device__ __forceinline__ double ldx(const double* a, int i) { return __ldcg(a + i); }

// D_theta x at (r, t, z) with the helical cross-term coefficients (ct1)
__device__ double d_theta(const AarArgs& A, const double (*C)[kMaxFDn + 1], const double* x, int r, int t, int z) {
  double s = 0;
  const int base = z * A.Nx * A.Ny + r;
  for (int q = 1; q <= A.F; ++q) {
    const int tp = wrap_idx(t + q, A.Ny, A.bcy), tm = wrap_idx(t - q, A.Ny, A.bcy);
    const double a = tp >= 0 ? ldx(x, base + tp * A.Nx) : 0.0, b = tm >= 0 ? ldx(x, base + tm * A.Nx) : 0.0;
    s += C[3][q] * (a - b);
  }
  return s;
}

// Lap_std x at point p (matrix-free, the arithmetic of the Hamiltonian kernels' Laplacian)
// (coefficients C: cr2, cr1, ct2, ct1, cz2, cz1 rows, staged in shared memory with 1/r and the theta scale)
// FT > 0: the FD half-width is FT at compile time, the loop is unrolled and every neighbour load
// is independent of the others (predicated at the walls), so a thread has them all in flight at
// once; FT = 0: half-width A.F at run time.
template <int FT>
__device__ __forceinline__ double lap_at(const AarArgs& A, const double (*C)[kMaxFDn + 1], const double* rinv, const double* thsc,
                                         const double* x, const double* vt, int p) {
  const int Nx = A.Nx, Ny = A.Ny, plane = Nx * Ny;
  const int r = p % Nx, t = (p / Nx) % Ny, z = p / plane;
  const int F = FT > 0 ? FT : A.F;
  const double xc = ldx(x, p);
  double s2 = C[0][0] * xc, s1 = 0, st2 = C[2][0] * xc, sz = C[4][0] * xc, sx = 0;
#pragma unroll
  for (int q = 1; q <= (FT > 0 ? FT : kMaxFDn); ++q) {
    if (FT == 0 && q > F) break;
    const double a = r + q < Nx ? ldx(x, p + q) : 0.0, b = r - q >= 0 ? ldx(x, p - q) : 0.0;
    const int tp = wrap_idx(t + q, Ny, A.bcy), tm = wrap_idx(t - q, Ny, A.bcy);
    const double c = tp >= 0 ? ldx(x, p + (tp - t) * Nx) : 0.0, d = tm >= 0 ? ldx(x, p + (tm - t) * Nx) : 0.0;
    const int zp = wrap_idx(z + q, A.Nz, A.bcz), zm = wrap_idx(z - q, A.Nz, A.bcz);
    const double e = zp >= 0 ? ldx(x, p + (zp - z) * plane) : 0.0, g = zm >= 0 ? ldx(x, p + (zm - z) * plane) : 0.0;
    s2 += C[0][q] * (a + b);
    s1 += C[1][q] * (a - b);
    st2 += C[2][q] * (c + d);
    sz += C[4][q] * (e + g);
    if (A.helical) {
      const double u = zp >= 0 ? ldx(vt, p + (zp - z) * plane) : 0.0, w = zm >= 0 ? ldx(vt, p + (zm - z) * plane) : 0.0;
      sx += C[5][q] * (u - w);
    }
  }
  return s2 + rinv[r] * s1 + thsc[r] * st2 + sz + sx;
}

// The AAR loop of src/aar.m:55-80.  Each iteration evaluates the residual at the current iterate
// and, on a Richardson iteration, writes the next iterate x + omega res into the other buffer in
// the same pass; one grid barrier then publishes both and the norm.  An Anderson iteration (every
// p-th) reduces the normal equations, solves them in block 0 and updates after two more barriers.
template <int FT>
__global__ void __launch_bounds__(256, 2) k_aar(const __grid_constant__ AarArgs A) {
  extern __shared__ double rtab[];                  // 1/r and theta scale per radial node (2 Nx)
  __shared__ double sh[32];
  __shared__ double gsh[kAarM * kAarM + 2 * kAarM];
  __shared__ double jA[64], jV[64], jcs[16];        // Anderson solve (block 0, warp 0)
  __shared__ double nred[8 * kNormal];              // normal-equation block sums (8 warps)
  __shared__ double C[6][kMaxFDn + 1];
  __shared__ double relres_s;
  if (threadIdx.x <= kMaxFDn) {
    const int q = threadIdx.x;
    C[0][q] = A.cr2[q]; C[1][q] = A.cr1[q]; C[2][q] = A.ct2[q]; C[3][q] = A.ct1[q]; C[4][q] = A.cz2[q]; C[5][q] = A.cz1[q];
  }
  for (int i = threadIdx.x; i < A.Nx; i += blockDim.x) {
    rtab[i] = A.rinv[i];
    rtab[A.Nx + i] = A.thsc[i];
  }
  __syncthreads();
  const double* rinv = rtab;
  const double* thsc = rtab + A.Nx;
  const int m = kAarM, N = A.N, nblk = gridDim.x;
  const int stride = gridDim.x * blockDim.x;
  const int tid0 = blockIdx.x * blockDim.x + threadIdx.x;
  double relres = 1 + A.tol;
  int count = 1;
  double* xc = A.x0;
  double* xn = A.x1;
  while (count <= A.maxit && relres > A.tol) {
    if (A.helical) {
      for (int p = tid0; p < N; p += stride) {
        const int r = p % A.Nx, t = (p / A.Nx) % A.Ny, z = p / (A.Nx * A.Ny);
        A.vt[p] = d_theta(A, C, xc, r, t, z);
      }
      if (!grid_sync(A.bar, A.status)) break;
    }
    // r = f - Lap x; res = dinv r; history columns; ||r||^2; Richardson step into the other buffer
    const int col = (count - 2 + m) % m;
    const bool anderson = count % A.p == 0;
    double s = 0;
    for (int p = tid0; p < N; p += stride) {
      const double rv = A.f[p] - lap_at<FT>(A, C, rinv, thsc, xc, A.vt, p);
      const double pv = A.dinv[p] * rv;
      const double xv = xc[p];
      s += rv * rv;
      if (count > 1) {
        A.DX[(size_t)col * N + p] = xv - A.xold[p];
        A.DF[(size_t)col * N + p] = pv - A.fold[p];
      }
      A.xold[p] = xv;
      A.fold[p] = pv;
      A.res[p] = pv;
      if (!anderson) xn[p] = xv + A.omega * pv;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) A.part[(count & 1) * nblk + blockIdx.x] = s;
    if (anderson) {
      // this block's share of the normal equations over its own points (written above): the
      // upper triangle of DF'DF and DF'res, kNormal sums reduced together
      double acc[kNormal];
#pragma unroll
      for (int k = 0; k < kNormal; ++k) acc[k] = 0;
      for (int p = tid0; p < N; p += stride) {
        double d[kAarM];
#pragma unroll
        for (int j = 0; j < kAarM; ++j) d[j] = A.DF[(size_t)j * N + p];
        const double rp = A.res[p];
        int k = 0;
#pragma unroll
        for (int i = 0; i < kAarM; ++i)
#pragma unroll
          for (int j = i; j < kAarM; ++j) acc[k++] += d[i] * d[j];
#pragma unroll
        for (int i = 0; i < kAarM; ++i) acc[k++] += d[i] * rp;
      }
      block_sum_many(acc, nred, A.part + 2 * nblk + (size_t)blockIdx.x * kNormal);
    }
    if (!grid_sync(A.bar, A.status)) break;
    relres = sqrt(sum_partials(A.part + (count & 1) * nblk, nblk, sh)) * A.nb;
    if (!(relres > A.tol)) break;   // x (= xold) is the converged iterate (aar.m:57-80)
    if (anderson) {
      if (blockIdx.x == 0) {
        __shared__ double tot[kNormal];
        for (int k = threadIdx.x; k < kNormal; k += blockDim.x) {
          double t = 0;
#pragma unroll 8
          for (int b = 0; b < nblk; ++b) t += __ldcg(A.part + 2 * nblk + (size_t)b * kNormal + k);
          tot[k] = t;
        }
        __syncthreads();
        // the full symmetric matrix (row-major) and the right-hand side for the solve
        if (threadIdx.x < m * m) {
          const int i = threadIdx.x / m, j = threadIdx.x % m, a = min(i, j), b = max(i, j);
          gsh[threadIdx.x] = tot[a * m - a * (a - 1) / 2 + (b - a)];
        } else if (threadIdx.x < m * m + m) {
          gsh[threadIdx.x] = tot[m * (m + 1) / 2 + (threadIdx.x - m * m)];
        }
        __syncthreads();
        if (threadIdx.x < 32) {
          pinv_solve_warp(gsh, jA, jV, jcs);        // gamma -> gsh[m*m + m ..]
          if (threadIdx.x < m) A.gam[threadIdx.x] = gsh[m * m + m + threadIdx.x];
        }
      }
      if (!grid_sync(A.bar, A.status)) break;
      double gam[kAarM];
      for (int i = 0; i < m; ++i) gam[i] = __ldcg(A.gam + i);
      for (int p = tid0; p < N; p += stride) {
        double u = xc[p] + A.beta * A.res[p];
        for (int i = 0; i < m; ++i) u -= (A.DX[(size_t)i * N + p] + A.beta * A.DF[(size_t)i * N + p]) * gam[i];
        xn[p] = u;
      }
      if (!grid_sync(A.bar, A.status)) break;
    }
    double* t = xc;
    xc = xn;
    xn = t;
    count++;
  }
  // the returned iterate is x_prev of the last residual evaluation (aar.m:77)
  for (int p = tid0; p < N; p += stride) A.phi[p] = A.xold[p];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *A.out_iters = min(count, A.maxit);
    *A.out_relres = relres;
  }
  (void)relres_s;
}

}  // namespace cx

namespace cx {

// AAR on device vectors: f (N) given, phi (N) initial guess when use_guess and result.
cx_status poisson_dev(cx_handle h, const double* d_f, double* d_phi, double tol, int32_t maxit, int32_t use_guess, int32_t* iters,
                      double* relres_out) {
  if (!h || !d_f || !d_phi) return CX_ERR_ARG;
  if (maxit < 1 || !(tol > 0)) { h->err = "cx_poisson: need maxit >= 1 and tol > 0"; return CX_ERR_ARG; }
  const int N = h->g.N, m = kAarM;
  // grid: resident blocks of 256 threads (cooperative launch)
  int dev = 0, nsm = 0, per_sm = 0;
  CX_TRY_CUDA(h, cudaGetDevice(&dev));
  CX_TRY_CUDA(h, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t dyn_smem = (size_t)2 * h->g.Nx * sizeof(double);
  // FD order 12 (the reference's default) has its own instance with the neighbour loop unrolled
  const void* kern = h->g.FDn == 6 ? (const void*)k_aar<6> : (const void*)k_aar<0>;
  CX_TRY_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, dyn_smem));
  if (per_sm < 1) { h->err = "cx_poisson: the AAR kernel does not fit on an SM"; return CX_ERR_CUDA; }
  // every block resident (cooperative launch), at most one point per thread
  const int nblocks = std::max(1, std::min(nsm * std::min(per_sm, 2), (N + 255) / 256));
  // workspace: x (two), vt, res, xold, fold, dinv (N each), DX, DF (N x m), 1/r and theta scale
  // (Nx each), per-block partials, Anderson weights, barrier word, outputs
  const size_t parts = (size_t)2 * nblocks + (size_t)nblocks * m * (m + 1);
  const size_t need = (size_t)N * 8 * (7 + 2 * m) + (size_t)h->g.Nx * 16 + parts * 8 + 8 * m + 16 * 256;
  if (h->pois_bytes < need) {
    cudaFree(h->d_pois);
    h->d_pois = nullptr;
    h->pois_bytes = 0;
    CX_TRY_CUDA(h, cudaMalloc(&h->d_pois, need));
    h->pois_bytes = need;
  }
  char* q = (char*)h->d_pois;
  auto take = [&](size_t bytes) { char* o = q; q += (bytes + 255) & ~(size_t)255; return (void*)o; };
  AarArgs A{};
  A.x0 = (double*)take((size_t)N * 8);
  A.x1 = (double*)take((size_t)N * 8);
  A.vt = (double*)take((size_t)N * 8);
  A.res = (double*)take((size_t)N * 8);
  A.xold = (double*)take((size_t)N * 8);
  A.fold = (double*)take((size_t)N * 8);
  double* dinv = (double*)take((size_t)N * 8);
  A.DX = (double*)take((size_t)N * 8 * m);
  A.DF = (double*)take((size_t)N * 8 * m);
  double* rinv = (double*)take((size_t)h->g.Nx * 8);
  double* thsc = (double*)take((size_t)h->g.Nx * 8);
  A.part = (double*)take(parts * 8);
  A.gam = (double*)take(8 * m);
  A.bar = (unsigned*)take(64);
  int* outs = (int*)take(64);
  double* outr = (double*)take(64);
  cudaStream_t st = h->stream;
  const unsigned gN = (unsigned)std::min(152 * 8, (N + 255) / 256);
  const cx_grid& G = h->grid;
  const GridDev& g = h->g;
  A.Nx = g.Nx; A.Ny = g.Ny; A.Nz = g.Nz; A.N = N; A.F = g.FDn; A.helical = g.helical; A.bcy = g.BCy; A.bcz = g.BCz;
  for (int k = 0; k <= kMaxFDn; ++k) {
    A.cr2[k] = h->coef.cr2[k]; A.cr1[k] = h->coef.cr1[k]; A.ct2[k] = h->coef.ct2[k];
    A.ct1[k] = h->coef.ct1[k]; A.cz2[k] = h->coef.cz2[k]; A.cz1[k] = h->coef.cz1[k];
  }
  {
    // the per-radial-node factors of the Laplacian (as the Hamiltonian kernels compute them)
    std::vector<double> ri(g.Nx), ts(g.Nx);
    for (int r = 0; r < g.Nx; ++r) {
      const double rr = g.xin + (double)r * g.dx;
      ri[r] = 1.0 / rr;
      ts[r] = g.helical ? g.twist * g.twist + 1.0 / (rr * rr) : 1.0 / (rr * rr);
    }
    CX_TRY_CUDA(h, cudaMemcpyAsync(rinv, ri.data(), g.Nx * 8, cudaMemcpyHostToDevice, st));
    CX_TRY_CUDA(h, cudaMemcpyAsync(thsc, ts.data(), g.Nx * 8, cudaMemcpyHostToDevice, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  }
  A.rinv = rinv;
  A.thsc = thsc;
  A.f = d_f;
  A.dinv = dinv;
  A.status = h->d_status;
  A.phi = d_phi;
  A.out_iters = outs;
  A.out_relres = outr;
  A.tol = tol;
  A.omega = 0.6;
  A.beta = 0.6;
  A.maxit = maxit;
  A.p = 6;
  // x0 = guess or ones (aar.m:51-53); history, sums and barrier cleared; ||f||
  if (use_guess) CX_TRY_CUDA(h, cudaMemcpyAsync(A.x0, d_phi, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
  else {
    std::vector<double> ones(N, 1.0);
    CX_TRY_CUDA(h, cudaMemcpyAsync(A.x0, ones.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  }
  CX_TRY_CUDA(h, cudaMemsetAsync(A.vt, 0, (size_t)N * 8, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.DX, 0, (size_t)N * 8 * m, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.DF, 0, (size_t)N * 8 * m, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.part, 0, parts * 8, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.bar, 0, 64, st));
  const double d0 = G.w2[0] / (G.dx * G.dx) + G.w2[0] / (G.dz * G.dz);
  k_pois_diag<<<gN, 256, 0, st>>>(dinv, G.Nx, N, G.xin, G.dx, d0, G.w2[0] / (G.dy * G.dy), G.twist * G.twist, G.cell_typ != 3);
  h->launches++;
  {
    std::vector<double> fh(N);
    CX_TRY_CUDA(h, cudaMemcpyAsync(fh.data(), d_f, (size_t)N * 8, cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    double nb2 = 0;
    for (double v : fh) nb2 += v * v;
    A.nb = 1.0 / std::sqrt(nb2);
  }
  void* args[] = {(void*)&A};
  CX_TRY_CUDA(h, cudaLaunchCooperativeKernel(kern, dim3(nblocks), dim3(256), args, dyn_smem, st));
  h->launches++;
  int it = 0, bst = 0;
  double rr = 0;
  CX_TRY_CUDA(h, cudaMemcpyAsync(&it, outs, sizeof(int), cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(&rr, outr, sizeof(double), cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(&bst, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  if (bst != 0) {
    CX_TRY_CUDA(h, cudaMemset(h->d_status, 0, sizeof(int)));
    h->err = "cx_poisson: a grid-barrier wait exceeded its limit (results of this call are invalid)";
    return CX_ERR_CUDA;
  }
  if (iters) *iters = it;
  if (relres_out) *relres_out = rr;
  if (rr > tol) {
    h->err = "cx_poisson: AAR reached maxit with relative residual " + std::to_string(rr);
    return CX_ERR_NOCONV;
  }
  return CX_OK;
}

// gamma = pinv(A) v for an m x m symmetric A, on the device (io layout of k_pois_pinv; m = 7, the
// AAR and Pulay history length)
cudaError_t launch_pinv_solve(double* io, int m, cudaStream_t st) {
  if (m != kAarM) return cudaErrorInvalidValue;
  k_pois_pinv<<<1, 32, 0, st>>>(io);
  return cudaGetLastError();
}

}  // namespace cx

extern "C" cx_status cx_poisson(cx_handle h, const double* f_host, double* phi_host, double tol, int32_t maxit, int32_t use_guess,
                                int32_t* iters, double* relres_out) {
  if (!h || !f_host || !phi_host) return CX_ERR_ARG;
  if (maxit < 1 || !(tol > 0)) { h->err = "cx_poisson: need maxit >= 1 and tol > 0"; return CX_ERR_ARG; }
  const size_t N = h->g.N;
  double *df = nullptr, *dphi = nullptr;
  cudaError_t e1 = cudaMalloc(&df, N * 8), e2 = cudaMalloc(&dphi, N * 8);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaFree(df);
    cudaFree(dphi);
    h->err = "cx_poisson: device vectors";
    return CX_ERR_NOMEM;
  }
  cx_status s = CX_OK;
  if (cudaMemcpy(df, f_host, N * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dphi, phi_host, N * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    h->err = "cx_poisson: copy in";
    s = CX_ERR_CUDA;
  }
  if (s == CX_OK) s = cx::poisson_dev(h, df, dphi, tol, maxit, use_guess, iters, relres_out);
  if ((s == CX_OK || s == CX_ERR_NOCONV) && cudaMemcpy(phi_host, dphi, N * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
    h->err = "cx_poisson: copy out";
    s = CX_ERR_CUDA;
  }
  cudaFree(df);
  cudaFree(dphi);
  return s;
}
