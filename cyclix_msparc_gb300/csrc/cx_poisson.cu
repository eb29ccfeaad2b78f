// Electrostatic Poisson solve: Alternating Anderson-Richardson (src/aar.m:1-74) on the
// assembled-equivalent operator Lap_std (src/initialization.m:734-740), applied matrix-free by
// the same fused stencil kernel as H*psi (k = 0, no potential, no projectors):
//     r = f - Lap_std x   is   out = 2 * (H x) + 1 * f   with H = -1/2 Lap.
// The reference preconditions with ILU(1e-5) (src/initialization.m:752); here the diagonal of
// Lap_std (Jacobi) is used, which keeps every step a streaming pass over HBM.  The Anderson
// least-squares step pinv(DF'DF) (DF' res) (aar.m:74) is solved on the device by a one-thread
// Jacobi eigen-decomposition of the m x m normal matrix with MATLAB's pinv tolerance.
#include <algorithm>
#include <cmath>

#include "cx_common.h"

namespace cx {

constexpr int kAarM = 7;   // Anderson history (poissonSolve.m:36)

struct PoisVecs {
  double2* x;     // iterate (complex storage for the stencil kernel, imaginary part 0)
  double2* r;     // residual f - A x
  double* f;
  double* res;    // preconditioned residual
  double* xold;
  double* fold;
  double* DX;     // N x m
  double* DF;     // N x m
  double* dinv;   // 1 / diag(Lap_std)
  double* zero;   // zero potential
  double* red;    // reductions: [0] = ||r||^2, [1..m*m] = DF'DF, [..m] = DF'res, gamma[m]
  BlockDev<double>* blk;
  int2* tab;
  StepScalars* sc;
};

__global__ void k_pois_diag(double* dinv, int Nx, int N, double xin, double dx, double d0, double dtheta0, double twist2, int helical) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double r = xin + (double)(i % Nx) * dx;
    const double th = helical ? (twist2 + 1.0 / (r * r)) : 1.0 / (r * r);
    dinv[i] = 1.0 / (d0 + th * dtheta0);
  }
}

__global__ void k_pois_prep(const double* f, double2* r, double2* x, const double* x0, int N, int use_guess) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    r[i] = make_double2(f[i], 0.0);
    x[i] = make_double2(use_guess ? x0[i] : 1.0, 0.0);
  }
}

__global__ void k_pois_copy_f(const double* f, double2* r, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) r[i] = make_double2(f[i], 0.0);
}

// res = dinv .* r ; ||r||^2 ; history columns (count > 1) ; Xold = x ; Fold = res
__global__ void k_pois_post(const double2* __restrict__ r, const double2* __restrict__ x, const double* __restrict__ dinv,
                            double* __restrict__ res, double* __restrict__ xold, double* __restrict__ fold, double* __restrict__ DXc,
                            double* __restrict__ DFc, int N, int store, double* __restrict__ nrm2) {
  double s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double rv = r[i].x;
    const double pv = dinv[i] * rv;
    const double xv = x[i].x;
    s += rv * rv;
    if (store) {
      DXc[i] = xv - xold[i];
      DFc[i] = pv - fold[i];
    }
    xold[i] = xv;
    fold[i] = pv;
    res[i] = pv;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    atomicAdd(nrm2, t);
  }
}

__global__ void k_pois_richardson(double2* x, const double* res, double omega, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) x[i].x += omega * res[i];
}

// normal matrix DF'DF (m x m) and DF'res (m): one CTA per output entry pair
__global__ void k_pois_gram(const double* __restrict__ DF, const double* __restrict__ res, int N, int m, double* __restrict__ out) {
  // blockIdx.x enumerates (i, j) with j <= m (j == m means res)
  const int i = blockIdx.x / (m + 1), j = blockIdx.x % (m + 1);
  const double* a = DF + (size_t)i * N;
  const double* b = j < m ? DF + (size_t)j * N : res;
  double s = 0;
  for (int k = threadIdx.x; k < N; k += blockDim.x) s += a[k] * b[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    if (j < m) out[i * m + j] = t; else out[m * m + i] = t;
  }
}

// gamma = pinv(A) * v for the symmetric m x m A (cyclic Jacobi eigen-decomposition, one thread)
__global__ void k_pois_pinv(double* __restrict__ io, int m) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
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

// x_new = x + beta res - (DX + beta DF) gamma
__global__ void k_pois_anderson(double2* x, const double* res, const double* DX, const double* DF, const double* gamma, double beta, int N,
                                int m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double u = x[i].x + beta * res[i];
    for (int k = 0; k < m; ++k) u -= (DX[(size_t)k * N + i] + beta * DF[(size_t)k * N + i]) * gamma[k];
    x[i].x = u;
  }
}

__global__ void k_pois_out(const double* xold, double* phi, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) phi[i] = xold[i];
}

}  // namespace cx

namespace cx {

// AAR on device vectors: f (N) given, phi (N) initial guess when use_guess and result.
cx_status poisson_dev(cx_handle h, const double* d_f, double* d_phi, double tol, int32_t maxit, int32_t use_guess, int32_t* iters,
                      double* relres_out) {
  if (!h || !d_f || !d_phi) return CX_ERR_ARG;
  if (maxit < 1 || !(tol > 0)) { h->err = "cx_poisson: need maxit >= 1 and tol > 0"; return CX_ERR_ARG; }
  const int N = h->g.N, m = kAarM, p = 6;
  const double omega = 0.6, beta = 0.6;
  // workspace
  const size_t need = (size_t)N * (16 * 2 + 8 * (5 + 2 * m + 1)) + 8 * (1 + m * m + 2 * m) + 4096;
  if (h->pois_bytes < need) {
    cudaFree(h->d_pois);
    h->d_pois = nullptr;
    h->pois_bytes = 0;
    CX_TRY_CUDA(h, cudaMalloc(&h->d_pois, need));
    h->pois_bytes = need;
  }
  char* q = (char*)h->d_pois;
  auto take = [&](size_t bytes) { char* o = q; q += (bytes + 255) & ~(size_t)255; return (void*)o; };
  PoisVecs v{};
  v.x = (double2*)take((size_t)N * 16);
  v.r = (double2*)take((size_t)N * 16);
  v.f = (double*)take((size_t)N * 8);
  v.res = (double*)take((size_t)N * 8);
  v.xold = (double*)take((size_t)N * 8);
  v.fold = (double*)take((size_t)N * 8);
  v.dinv = (double*)take((size_t)N * 8);
  v.zero = (double*)take((size_t)N * 8);
  v.DX = (double*)take((size_t)N * 8 * m);
  v.DF = (double*)take((size_t)N * 8 * m);
  v.red = (double*)take(8 * (1 + m * m + 2 * m));
  v.blk = (BlockDev<double>*)take(sizeof(BlockDev<double>));
  v.tab = (int2*)take(sizeof(int2));
  v.sc = (StepScalars*)take(sizeof(StepScalars));
  cudaStream_t st = h->stream;
  const unsigned gN = (unsigned)std::min(152 * 8, (N + 255) / 256);
  // operator descriptors: k = 0, zero potential
  BlockDev<double> bd{};
  bd.buf[0] = v.x;
  bd.buf[1] = v.r;
  bd.veff = v.zero;
  bd.ph_tl = bd.ph_tr = bd.ph_zl = bd.ph_zr = make_double2(1, 0);
  bd.Ns = 1;
  const int2 tab = make_int2(0, 0);
  const StepScalars sc{2.0, 0.0, 1.0, 0.0};
  CX_TRY_CUDA(h, cudaMemcpyAsync(v.blk, &bd, sizeof(bd), cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(v.tab, &tab, sizeof(tab), cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(v.sc, &sc, sizeof(sc), cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(v.zero, 0, (size_t)N * 8, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(v.f, d_f, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
  if (use_guess) CX_TRY_CUDA(h, cudaMemcpyAsync(v.res, d_phi, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(v.DX, 0, (size_t)N * 8 * m, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(v.DF, 0, (size_t)N * 8 * m, st));
  const cx_grid& G = h->grid;
  const double d0 = G.w2[0] / (G.dx * G.dx) + G.w2[0] / (G.dz * G.dz);
  k_pois_diag<<<gN, 256, 0, st>>>(v.dinv, G.Nx, N, G.xin, G.dx, d0, G.w2[0] / (G.dy * G.dy), G.twist * G.twist,
                                  G.cell_typ != 3);
  k_pois_prep<<<gN, 256, 0, st>>>(v.f, v.r, v.x, v.res, N, use_guess);
  h->launches += 2;
  // ||f||
  double nb2 = 0;
  {
    CX_TRY_CUDA(h, cudaMemsetAsync(v.red, 0, 8, st));
    // reuse the post kernel on r = f with x = guess to get ||f||^2 (history not stored)
    k_pois_post<<<gN, 256, 0, st>>>(v.r, v.x, v.dinv, v.res, v.xold, v.fold, v.DX, v.DF, N, 0, v.red);
    h->launches++;
    CX_TRY_CUDA(h, cudaMemcpyAsync(&nb2, v.red, 8, cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  }
  const double nb = 1.0 / std::sqrt(nb2);
  double relres = 1 + tol;
  int count = 1;
  cx_status s;
  while (count <= maxit && relres > tol) {
    // r = f - Lap x
    k_pois_copy_f<<<gN, 256, 0, st>>>(v.f, v.r, N);
    h->launches++;
    s = fused_step<double>(h, v.blk, v.sc, 1, v.tab, 1, 0, true, nullptr, false, 0.0);
    if (s != CX_OK) return s;
    CX_TRY_CUDA(h, cudaMemsetAsync(v.red, 0, 8, st));
    const int col = (count - 2) % m;
    k_pois_post<<<gN, 256, 0, st>>>(v.r, v.x, v.dinv, v.res, v.xold, v.fold, v.DX + (size_t)std::max(col, 0) * N,
                                    v.DF + (size_t)std::max(col, 0) * N, N, count > 1 ? 1 : 0, v.red);
    h->launches++;
    double r2 = 0;
    CX_TRY_CUDA(h, cudaMemcpyAsync(&r2, v.red, 8, cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    relres = std::sqrt(r2) * nb;
    if (!(relres > tol)) break;   // x (= Xold) is the converged iterate (aar.m:57-80)
    if (count % p != 0) {
      k_pois_richardson<<<gN, 256, 0, st>>>(v.x, v.res, omega, N);
      h->launches++;
    } else {
      k_pois_gram<<<m * (m + 1), 256, 0, st>>>(v.DF, v.res, N, m, v.red + 1);
      k_pois_pinv<<<1, 32, 0, st>>>(v.red + 1, m);
      k_pois_anderson<<<gN, 256, 0, st>>>(v.x, v.res, v.DX, v.DF, v.red + 1 + m * m + m, beta, N, m);
      h->launches += 3;
    }
    CX_TRY_CUDA(h, cudaGetLastError());
    count++;
  }
  // the returned iterate is x_prev of the last residual evaluation (aar.m:77)
  k_pois_out<<<gN, 256, 0, st>>>(v.xold, d_phi, N);
  h->launches++;
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  if (iters) *iters = std::min(count, maxit);
  if (relres_out) *relres_out = relres;
  if (relres > tol) {
    h->err = "cx_poisson: AAR reached maxit with relative residual " + std::to_string(relres);
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
