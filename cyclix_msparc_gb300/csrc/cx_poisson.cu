// Electrostatic Poisson solve: Alternating Anderson-Richardson (src/aar.m:1-74) on the
// assembled-equivalent operator Lap_std (src/initialization.m:734-740), applied matrix-free:
//   cyclic:  (DL11 + DG1) x + R2inv x DL22^T + x DL33^T,  helical adds x DL22^T and (x DG2^T) DG3^T
// with real coefficients (k = 0) and the boundary conditions of the grid.
// The reference preconditions with ILU(1e-5) (src/initialization.m:752); here the diagonal of
// Lap_std (Jacobi) is used, which keeps every step a streaming pass.  The Anderson least-squares
// step pinv(DF'DF) (DF' res) (aar.m:74) is solved on the device by a one-thread Jacobi
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

// gamma = pinv(A) v for the symmetric m x m A in io (A row-major, then v; gamma written after v):
// cyclic Jacobi eigen-decomposition by one thread, MATLAB's pinv tolerance
__device__ __noinline__ void pinv_solve_1t(double* __restrict__ io, int m) {
  double A[kAarM][kAarM], V[kAarM][kAarM], v[kAarM];
  for (int i = 0; i < m; ++i) {
    v[i] = io[m * m + i];
    for (int j = 0; j < m; ++j) { A[i][j] = io[i * m + j]; V[i][j] = i == j ? 1.0 : 0.0; }
  }
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0;
    for (int i = 0; i < m; ++i) for (int j = i + 1; j < m; ++j) off += A[i][j] * A[i][j];
    if (off < 1e-300) break;
    for (int p = 0; p < m; ++p) {
      for (int q = p + 1; q < m; ++q) {
        if (fabs(A[p][q]) < 1e-300) continue;
        const double th = (A[q][q] - A[p][p]) / (2 * A[p][q]);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
        const double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < m; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
    }
  }
  double nrm = 0;
  for (int i = 0; i < m; ++i) nrm = fmax(nrm, fabs(A[i][i]));
  const double tol = m * nrm * 2.220446049250313e-16;   // MATLAB pinv: max(size(A)) * norm(A) * eps
  double g[kAarM];
  for (int i = 0; i < m; ++i) g[i] = 0;
  for (int k = 0; k < m; ++k) {
    if (fabs(A[k][k]) <= tol) continue;
    double c = 0;
    for (int i = 0; i < m; ++i) c += V[i][k] * v[i];
    c /= A[k][k];
    for (int i = 0; i < m; ++i) g[i] += V[i][k] * c;
  }
  for (int i = 0; i < m; ++i) io[m * m + m + i] = g[i];
}

__global__ void k_pois_pinv(double* __restrict__ io, int m) {
  if (threadIdx.x == 0 && blockIdx.x == 0) pinv_solve_1t(io, m);
}

// ---------------------------------------------------------------------------- persistent AAR
struct AarArgs {
  int Nx, Ny, Nz, N, F, helical, bcy, bcz;
  double xin, dx, twist;
  double cr2[kMaxFDn + 1], cr1[kMaxFDn + 1], ct2[kMaxFDn + 1], ct1[kMaxFDn + 1], cz2[kMaxFDn + 1], cz1[kMaxFDn + 1];
  const double* f;
  const double* dinv;
  double* x;          // iterate
  double* vt;         // helical: D_theta x
  double* res;        // preconditioned residual
  double* xold;
  double* fold;
  double* DX;         // N x m
  double* DF;         // N x m
  double* red;        // [0,1] ||r||^2 (by iteration parity), [2 .. 2+m*m+2m) normal matrix, DF'res, gamma
  unsigned* bar;      // [0] arrivals, [1] generation
  int* status;        // 1 when a barrier wait ran out
  double* phi;        // result
  int* out_iters;
  double* out_relres;
  double tol, nb, omega, beta;
  int maxit, p;
};

// Grid barrier of a cooperative launch (every block resident): arrival counter and generation
// word in global memory; the wait is bounded (about a second), after which *status is set and
// false is returned to every thread of the block.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* status) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const long long t_end = clock64() + (1LL << 31);
      while (*gen == g) {
        if (clock64() > t_end) { ok = 0; atomicExch(status, 1); break; }
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
// (coefficients C: cr2, cr1, ct2, ct1, cz2, cz1 rows, staged in shared memory)
__device__ double lap_at(const AarArgs& A, const double (*C)[kMaxFDn + 1], const double* x, const double* vt, int p) {
  const int Nx = A.Nx, Ny = A.Ny, plane = Nx * Ny;
  const int r = p % Nx, t = (p / Nx) % Ny, z = p / plane;
  const double xc = ldx(x, p);
  const double rr = A.xin + (double)r * A.dx;
  const double inv_r = 1.0 / rr;
  const double th_scale = A.helical ? A.twist * A.twist + 1.0 / (rr * rr) : 1.0 / (rr * rr);
  double s2 = C[0][0] * xc, s1 = 0, st2 = C[2][0] * xc, sz = C[4][0] * xc, sx = 0;
  for (int q = 1; q <= A.F; ++q) {
    const double a = r + q < Nx ? ldx(x, p + q) : 0.0, b = r - q >= 0 ? ldx(x, p - q) : 0.0;
    s2 += C[0][q] * (a + b);
    s1 += C[1][q] * (a - b);
    const int tp = wrap_idx(t + q, Ny, A.bcy), tm = wrap_idx(t - q, Ny, A.bcy);
    const double c = tp >= 0 ? ldx(x, p + (tp - t) * Nx) : 0.0, d = tm >= 0 ? ldx(x, p + (tm - t) * Nx) : 0.0;
    st2 += C[2][q] * (c + d);
    const int zp = wrap_idx(z + q, A.Nz, A.bcz), zm = wrap_idx(z - q, A.Nz, A.bcz);
    const double e = zp >= 0 ? ldx(x, p + (zp - z) * plane) : 0.0, g = zm >= 0 ? ldx(x, p + (zm - z) * plane) : 0.0;
    sz += C[4][q] * (e + g);
    if (A.helical) {
      const double u = zp >= 0 ? ldx(vt, p + (zp - z) * plane) : 0.0, w = zm >= 0 ? ldx(vt, p + (zm - z) * plane) : 0.0;
      sx += C[5][q] * (u - w);
    }
  }
  return s2 + inv_r * s1 + th_scale * st2 + sz + sx;
}

__global__ void __launch_bounds__(256, 2) k_aar(const __grid_constant__ AarArgs A) {
  __shared__ double sh[32];
  __shared__ double gsh[kAarM * kAarM + 2 * kAarM];
  __shared__ double C[6][kMaxFDn + 1];
  if (threadIdx.x <= kMaxFDn) {
    const int q = threadIdx.x;
    C[0][q] = A.cr2[q]; C[1][q] = A.cr1[q]; C[2][q] = A.ct2[q]; C[3][q] = A.ct1[q]; C[4][q] = A.cz2[q]; C[5][q] = A.cz1[q];
  }
  __syncthreads();
  const int m = kAarM, N = A.N;
  const int stride = gridDim.x * blockDim.x;
  const int tid0 = blockIdx.x * blockDim.x + threadIdx.x;
  double relres = 1 + A.tol;
  int count = 1;
  bool alive = true;
  while (alive && count <= A.maxit && relres > A.tol) {
    if (A.helical) {
      for (int p = tid0; p < N; p += stride) {
        const int r = p % A.Nx, t = (p / A.Nx) % A.Ny, z = p / (A.Nx * A.Ny);
        A.vt[p] = d_theta(A, C, A.x, r, t, z);
      }
      if (!grid_barrier(A.bar, A.status)) { alive = false; break; }
    }
    // r = f - Lap x; res = dinv r; history columns; ||r||^2
    const int col = (count - 2 + m) % m;
    double s = 0;
    for (int p = tid0; p < N; p += stride) {
      const double rv = A.f[p] - lap_at(A, C, A.x, A.vt, p);
      const double pv = A.dinv[p] * rv;
      const double xv = A.x[p];
      s += rv * rv;
      if (count > 1) {
        A.DX[(size_t)col * N + p] = xv - A.xold[p];
        A.DF[(size_t)col * N + p] = pv - A.fold[p];
      }
      A.xold[p] = xv;
      A.fold[p] = pv;
      A.res[p] = pv;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) atomicAdd(A.red + (count & 1), s);
    if (!grid_barrier(A.bar, A.status)) { alive = false; break; }
    relres = sqrt(__ldcg(A.red + (count & 1))) * A.nb;
    if (blockIdx.x == 0 && threadIdx.x == 0) A.red[(count + 1) & 1] = 0.0;    // next iteration's accumulator
    if (!(relres > A.tol)) break;   // x (= xold) is the converged iterate (aar.m:57-80)
    if (count % A.p != 0) {
      for (int p = tid0; p < N; p += stride) A.x[p] += A.omega * A.res[p];
    } else {
      // normal matrix DF'DF and DF'res (block partial sums, one row of it at a time), pinv by one
      // thread of block 0 (gamma published in red), then the update
      for (int i = 0; i < m; ++i) {
        double acc[kAarM + 1];
        for (int j = 0; j <= m; ++j) acc[j] = 0;
        for (int p = tid0; p < N; p += stride) {
          const double di = A.DF[(size_t)i * N + p];
          for (int j = 0; j < m; ++j) acc[j] += di * A.DF[(size_t)j * N + p];
          acc[m] += di * A.res[p];
        }
        for (int j = 0; j <= m; ++j) {
          const double t = block_sum(acc[j], sh);
          if (threadIdx.x == 0) atomicAdd(A.red + 2 + (j < m ? i * m + j : m * m + i), t);
        }
      }
      if (!grid_barrier(A.bar, A.status)) { alive = false; break; }
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int k = 0; k < m * m + m; ++k) {
          gsh[k] = __ldcg(A.red + 2 + k);
          A.red[2 + k] = 0.0;                       // cleared for the next Anderson step
        }
        pinv_solve_1t(gsh, m);                      // gamma -> gsh[m*m + m ..]
        for (int i = 0; i < m; ++i) A.red[2 + m * m + m + i] = gsh[m * m + m + i];
      }
      if (!grid_barrier(A.bar, A.status)) { alive = false; break; }
      double gam[kAarM];
      for (int i = 0; i < m; ++i) gam[i] = __ldcg(A.red + 2 + m * m + m + i);
      for (int p = tid0; p < N; p += stride) {
        double u = A.x[p] + A.beta * A.res[p];
        for (int i = 0; i < m; ++i) u -= (A.DX[(size_t)i * N + p] + A.beta * A.DF[(size_t)i * N + p]) * gam[i];
        A.x[p] = u;
      }
    }
    if (!grid_barrier(A.bar, A.status)) { alive = false; break; }
    count++;
  }
  // the returned iterate is x_prev of the last residual evaluation (aar.m:77)
  for (int p = tid0; p < N; p += stride) A.phi[p] = A.xold[p];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *A.out_iters = min(count, A.maxit);
    *A.out_relres = relres;
  }
}

}  // namespace cx

namespace cx {

// AAR on device vectors: f (N) given, phi (N) initial guess when use_guess and result.
cx_status poisson_dev(cx_handle h, const double* d_f, double* d_phi, double tol, int32_t maxit, int32_t use_guess, int32_t* iters,
                      double* relres_out) {
  if (!h || !d_f || !d_phi) return CX_ERR_ARG;
  if (maxit < 1 || !(tol > 0)) { h->err = "cx_poisson: need maxit >= 1 and tol > 0"; return CX_ERR_ARG; }
  const int N = h->g.N, m = kAarM;
  // workspace: x, vt, res, xold, fold, dinv (N each), DX, DF (N x m), reductions, barrier, outputs
  const size_t need = (size_t)N * 8 * (6 + 2 * m) + 8 * (2 + m * m + 2 * m) + 4096;
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
  A.x = (double*)take((size_t)N * 8);
  A.vt = (double*)take((size_t)N * 8);
  A.res = (double*)take((size_t)N * 8);
  A.xold = (double*)take((size_t)N * 8);
  A.fold = (double*)take((size_t)N * 8);
  double* dinv = (double*)take((size_t)N * 8);
  A.DX = (double*)take((size_t)N * 8 * m);
  A.DF = (double*)take((size_t)N * 8 * m);
  A.red = (double*)take(8 * (2 + m * m + 2 * m));
  A.bar = (unsigned*)take(64);
  int* outs = (int*)take(64);
  double* outr = (double*)take(64);
  cudaStream_t st = h->stream;
  const unsigned gN = (unsigned)std::min(152 * 8, (N + 255) / 256);
  const cx_grid& G = h->grid;
  const GridDev& g = h->g;
  A.Nx = g.Nx; A.Ny = g.Ny; A.Nz = g.Nz; A.N = N; A.F = g.FDn; A.helical = g.helical; A.bcy = g.BCy; A.bcz = g.BCz;
  A.xin = g.xin; A.dx = g.dx; A.twist = g.twist;
  for (int k = 0; k <= kMaxFDn; ++k) {
    A.cr2[k] = h->coef.cr2[k]; A.cr1[k] = h->coef.cr1[k]; A.ct2[k] = h->coef.ct2[k];
    A.ct1[k] = h->coef.ct1[k]; A.cz2[k] = h->coef.cz2[k]; A.cz1[k] = h->coef.cz1[k];
  }
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
  if (use_guess) CX_TRY_CUDA(h, cudaMemcpyAsync(A.x, d_phi, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
  else {
    std::vector<double> ones(N, 1.0);
    CX_TRY_CUDA(h, cudaMemcpyAsync(A.x, ones.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  }
  CX_TRY_CUDA(h, cudaMemsetAsync(A.vt, 0, (size_t)N * 8, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.DX, 0, (size_t)N * 8 * m, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.DF, 0, (size_t)N * 8 * m, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.red, 0, 8 * (2 + m * m + 2 * m), st));
  CX_TRY_CUDA(h, cudaMemsetAsync(A.bar, 0, 64, st));
  const double d0 = G.w2[0] / (G.dx * G.dx) + G.w2[0] / (G.dz * G.dz);
  k_pois_diag<<<gN, 256, 0, st>>>(dinv, G.Nx, N, G.xin, G.dx, d0, G.w2[0] / (G.dy * G.dy), G.twist * G.twist, G.cell_typ != 3);
  h->launches++;
  {
    // ||f||^2 by cuBLAS-free reduction: reuse the red slot 0
    std::vector<double> fh(N);
    CX_TRY_CUDA(h, cudaMemcpyAsync(fh.data(), d_f, (size_t)N * 8, cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    double nb2 = 0;
    for (double v : fh) nb2 += v * v;
    A.nb = 1.0 / std::sqrt(nb2);
  }
  // one resident grid: as many blocks as fit on the device at once (cooperative launch)
  int dev = 0, nsm = 0, per_sm = 0;
  CX_TRY_CUDA(h, cudaGetDevice(&dev));
  CX_TRY_CUDA(h, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  CX_TRY_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_aar, 256, 0));
  const int nblocks = std::max(1, std::min(nsm * std::max(1, per_sm), (N + 255) / 256));
  void* args[] = {(void*)&A};
  CX_TRY_CUDA(h, cudaLaunchCooperativeKernel((const void*)k_aar, dim3(nblocks), dim3(256), args, 0, st));
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

// gamma = pinv(A) v for an m x m symmetric A, on the device (io layout of k_pois_pinv)
cudaError_t launch_pinv_solve(double* io, int m, cudaStream_t st) {
  k_pois_pinv<<<1, 32, 0, st>>>(io, m);
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
