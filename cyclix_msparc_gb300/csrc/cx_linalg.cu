// Subspace part of the CheFSI step (src/eigSolver.m:47-124) and host <-> device transfers.
//
//  * spectral bounds: a batched Lanczos iteration in the W inner product (the operator is
//    self-adjoint in it away from the two radial end rows), the extreme Ritz values of the
//    tridiagonal matrix found by Sturm-sequence bisection on the GPU; it stands in for
//    eigs(Hfun,N,1,'lr'/'sr') of src/eigSolver.m:47-67 (bup = 1.01 lambda_max, a0 = lambda_min - 0.1);
//  * Rayleigh-Ritz per block: Gram G = X^H X, M = X^H (H X) and the W-Gram X^H W X (complex128:
//    cuBLAS ZGEMM; complex64: the tcgen05 3xTF32 kernels of cx_tcgen05.cu, FP64 sums of FP32
//    partials), FP64 Cholesky G = R^H R and the pencil A = G^-1 M, whose eigenvalues are those of
//    the reference's Hs = R A R^-1 (orth + psi'*H*psi of :99-104, in a basis of the same span);
//    the eigenpairs of A (:110) through the W-similar, nearly Hermitian T = U_w A U_w^-1 and a
//    fixed-point refinement (restarted when it stalls), the general FP64 solver as the last
//    resort; real part and ascending sort (:111-116), rotation psi = X c (:119) and
//    W-normalisation of the columns (:122-124).
#include <algorithm>
#include <cmath>
#include <complex>
#include <numeric>
#include <thread>

#include "cx_common.h"

namespace cx {

__global__ void k_d2f(const double2* __restrict__ a, float2* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void k_f2d(const float2* __restrict__ a, double2* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = make_double2((double)a[i].x, (double)a[i].y);
}

// ||X - I||_F^2 of an n x n complex matrix into *out (one CTA)
__global__ void k_dist_identity2(const double2* __restrict__ X, int n, double* __restrict__ out) {
  double t = 0;
  const size_t n2 = (size_t)n * n;
  for (size_t e = threadIdx.x; e < n2; e += blockDim.x) {
    const double re = X[e].x - ((e % (size_t)(n + 1)) == 0 ? 1.0 : 0.0);
    t += re * re + X[e].y * X[e].y;
  }
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) a += sh[k];
    *out = a;
  }
}

__global__ void k_r2d(const float* __restrict__ a, double* __restrict__ b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = (double)a[i];
}

static unsigned grid_for(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16); }

static cx_status ensure(cx_handle h, void** p, size_t* cap, size_t bytes) {
  if (*cap >= bytes) return CX_OK;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    h->err = std::string("workspace allocation of ") + std::to_string(bytes) + " B: " + cudaGetErrorString(e);
    return CX_ERR_NOMEM;
  }
  *cap = bytes;
  return CX_OK;
}

// ------------------------------------------------------------------ W-normalisation (:122-124)
// The complex64 kernels read a float copy of W: a double-to-float conversion per element runs on
// GB300's narrow FP64 pipe.  Columns are indexed by blockIdx.y (no per-element division).
template <typename R> struct WOf;
template <> struct WOf<float> { using T = float; };
template <> struct WOf<double> { using T = double; };

template <typename R>
__global__ void k_colnorm_w(const cplx<R>* __restrict__ X, const typename WOf<R>::T* __restrict__ W, int N, double* __restrict__ out) {
  const cplx<R>* x = X + (size_t)blockIdx.x * N;
  // per-thread compensated sum in the working precision, then the block reduction in double
  R s = 0, comp = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const cplx<R> v = x[i];
    const R term = W[i] * (v.x * v.x + v.y * v.y) - comp;
    const R t = s + term;
    comp = (t - s) - term;
    s = t;
  }
  double acc = (double)s;
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    out[blockIdx.x] = 1.0 / sqrt(t);
  }
}
template <typename R>
__global__ void k_colscale(cplx<R>* __restrict__ X, int N, int ncol, const double* __restrict__ sc) {
  for (int col = blockIdx.y; col < ncol; col += gridDim.y) {
    const R s = (R)sc[col];
    cplx<R>* x = X + (size_t)col * N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
      x[i].x *= s;
      x[i].y *= s;
    }
  }
}
template <typename R>
__global__ void k_wscale(const cplx<R>* __restrict__ X, cplx<R>* __restrict__ Y, const typename WOf<R>::T* __restrict__ W, int N, int n) {
  for (int col = blockIdx.y; col < n; col += gridDim.y) {
    const cplx<R>* x = X + (size_t)col * N;
    cplx<R>* y = Y + (size_t)col * N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
      const R w = W[i];
      y[i].x = x[i].x * w;
      y[i].y = x[i].y * w;
    }
  }
}
static dim3 col_grid(int N, int n) {
  return dim3((unsigned)std::min(64, (N + 255) / 256), (unsigned)std::min(n, 65535));
}

// gather columns: out[:, j] = in[:, perm[j]]
__global__ void k_gather_cols(const double2* __restrict__ in, double2* __restrict__ out, int n, const int* __restrict__ perm) {
  const size_t tot = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t j = i / n, r = i % n;
    out[i] = in[(size_t)perm[j] * n + r];
  }
}

// ------------------------------------------------------------------ subspace eigensolver kernels
// WX = W .* X (column-major N x n)
// X += I
__global__ void k_add_identity(double2* __restrict__ X, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) X[(size_t)i * n + i].x += 1.0;
}
// Th = (T + T^H) / 2
__global__ void k_herm_part(const double2* __restrict__ T, double2* __restrict__ Th, int n) {
  const size_t tot = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = i % n, c = i / n;
    const double2 a = T[i], b = T[r * n + c];
    Th[i] = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
  }
}
// split B into its diagonal d and the off-diagonal part E (in place); Z = 0
__global__ void k_split_diag(double2* __restrict__ B, double2* __restrict__ d, double2* __restrict__ Z, int n) {
  const size_t tot = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = i % n, c = i / n;
    if (r == c) { d[r] = B[i]; B[i] = make_double2(0, 0); }
    Z[i] = make_double2(0, 0);
  }
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double den = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}
// one fixed-point sweep of B X = X Lambda with X = I + Z (Z zero on the diagonal), B = diag(d) + E:
//   lambda_j = d_j + (E Z)_jj ,  Zn_kj = (E_kj + (E Z)_kj) / (lambda_j - d_k)   (k != j)
// and dmax = max |Zn - Z| (a non-negative double compared through its bit pattern)
// (EZ in complex128, or in complex64 from the FP32-accurate tensor-core product of the mixed path)
template <typename V>
__global__ void k_sylv_update(const double2* __restrict__ E, const V* __restrict__ EZ, const double2* __restrict__ d,
                              const double2* __restrict__ Z, double2* __restrict__ Zn, int n, unsigned long long* __restrict__ dmax) {
  const size_t tot = (size_t)n * n;
  double m = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t k = i % n, j = i / n;
    double2 v = make_double2(0, 0);
    if (k != j) {
      const V ejj = EZ[j * n + j];
      const double2 lam = make_double2(d[j].x + (double)ejj.x, d[j].y + (double)ejj.y);
      v = cdiv(make_double2(E[i].x + (double)EZ[i].x, E[i].y + (double)EZ[i].y), make_double2(lam.x - d[k].x, lam.y - d[k].y));
    }
    Zn[i] = v;
    const double dd = fmax(fabs(v.x - Z[i].x), fabs(v.y - Z[i].y));
    m = (dd == dd) ? fmax(m, dd) : INFINITY;      // NaN marks divergence
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(dmax, (unsigned long long)__double_as_longlong(m));
}
// eigenvalues lambda_j = d_j + (E Z)_jj and eigenvectors X = I + Z (in place of Z)
__global__ void k_sylv_finish(const double2* __restrict__ EZ, const double2* __restrict__ d, double2* __restrict__ Z,
                              double2* __restrict__ lam, int n) {
  const size_t tot = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t k = i % n, j = i / n;
    if (k == j) {
      Z[i] = make_double2(1.0, 0.0);
      lam[j] = make_double2(d[j].x + EZ[i].x, d[j].y + EZ[i].y);
    }
  }
}

// Gy <- D^-1/2 Gy D^-1/2 (unit diagonal) for the rotation check
__global__ void k_unit_diag(double2* __restrict__ G, int n) {
  const size_t tot = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = i % n, c = i / n;
    const double d = sqrt(G[r * n + r].x * G[c * n + c].x);
    if (r != c) G[i] = make_double2(G[i].x / d, G[i].y / d);
  }
}
__global__ void k_unit_diag_fix(double2* __restrict__ G, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) G[(size_t)i * n + i] = make_double2(1.0, 0.0);
}
// smallest |R_jj| of a Cholesky factor (one CTA)
__global__ void k_min_diag(const double2* __restrict__ R, int n, double* __restrict__ out) {
  double m = 1e300;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = fabs(R[(size_t)i * n + i].x);
    m = (v == v) ? fmin(m, v) : 0.0;
  }
  for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 1e300;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmin(t, red[k]);
    *out = t;
  }
}
// eigenvalues of the Hermitian part (real) as complex values
__global__ void k_real_to_complex(const double* __restrict__ a, double2* __restrict__ b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = make_double2(a[i], 0.0);
}

// ------------------------------------------------------------------ batched Lanczos (W inner product)
// Per block b the vectors live at v + b*N etc.; scalars alpha[j*nblk+b], beta2[j*nblk+b].
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}
template <typename R>
__global__ void k_lz_init(cplx<R>* v, cplx<R>* vprev, int N, int nblk, uint32_t seed) {
  const size_t tot = (size_t)N * nblk;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t b = (uint32_t)(i / N);
    const uint32_t u = hash32((uint32_t)(i % N) * 2654435761u ^ hash32(seed + 7919u * (b + 1)));
    v[i].x = (R)((u >> 8) * (1.0 / 16777216.0));
    v[i].y = 0;
    vprev[i].x = 0;
    vprev[i].y = 0;
  }
}
// acc[b] += sum_n W_n Re(conj(a_n) b_n)
template <typename R>
__global__ void k_lz_dot(const cplx<R>* __restrict__ a, const cplx<R>* __restrict__ bv, const double* __restrict__ W, int N,
                         double* __restrict__ acc) {
  const int b = blockIdx.y;
  const cplx<R>* x = a + (size_t)b * N;
  const cplx<R>* y = bv + (size_t)b * N;
  double s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    s += W[i] * ((double)x[i].x * y[i].x + (double)x[i].y * y[i].y);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    atomicAdd(acc + b, t);
  }
}
// w = w - alpha v - beta vprev ; beta2_next += ||w||_W^2
template <typename R>
__global__ void k_lz_update(cplx<R>* __restrict__ w, const cplx<R>* __restrict__ v, const cplx<R>* __restrict__ vprev,
                            const double* __restrict__ W, int N, const double* __restrict__ alpha, const double* __restrict__ beta2,
                            double* __restrict__ beta2_next) {
  const int b = blockIdx.y;
  const double al = alpha[b];
  const double be = beta2 ? sqrt(fmax(beta2[b], 0.0)) : 0.0;
  cplx<R>* x = w + (size_t)b * N;
  const cplx<R>* v0 = v + (size_t)b * N;
  const cplx<R>* v1 = vprev + (size_t)b * N;
  double s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    cplx<R> t = x[i];
    t.x = (R)((double)t.x - al * v0[i].x - be * v1[i].x);
    t.y = (R)((double)t.y - al * v0[i].y - be * v1[i].y);
    x[i] = t;
    s += W[i] * ((double)t.x * t.x + (double)t.y * t.y);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    atomicAdd(beta2_next + b, t);
  }
}
// vprev = v ; v = w / sqrt(beta2) (zero when the iteration broke down)
template <typename R>
__global__ void k_lz_shift(const cplx<R>* __restrict__ w, cplx<R>* __restrict__ v, cplx<R>* __restrict__ vprev, int N,
                           const double* __restrict__ beta2) {
  const int b = blockIdx.y;
  const double bb = beta2[b];
  const double inv = bb > 1e-200 ? 1.0 / sqrt(bb) : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)b * N + i;
    vprev[k] = v[k];
    cplx<R> t = w[k];
    t.x = (R)(t.x * inv);
    t.y = (R)(t.y * inv);
    v[k] = t;
  }
}
// normalise the start vectors: v /= ||v||_W
template <typename R>
__global__ void k_lz_norm0(cplx<R>* __restrict__ v, int N, const double* __restrict__ n2) {
  const int b = blockIdx.y;
  const double inv = 1.0 / sqrt(n2[b]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)b * N + i;
    v[k].x = (R)(v[k].x * inv);
    v[k].y = (R)(v[k].y * inv);
  }
}
// Extreme eigenvalues of the K x K Lanczos tridiagonal of each block by Sturm bisection.
__device__ int sturm_count(const double* a, const double* b2, int K, int nblk, int blk, double x) {
  int cnt = 0;
  double d = 1.0;
  for (int j = 0; j < K; ++j) {
    const double off = j == 0 ? 0.0 : b2[(size_t)j * nblk + blk] / d;
    d = a[(size_t)j * nblk + blk] - x - off;
    if (fabs(d) < 1e-300) d = -1e-300;
    if (d < 0) ++cnt;
  }
  return cnt;
}
__global__ void k_tridiag_extremes(const double* __restrict__ alpha, const double* __restrict__ beta2, int K, int nblk,
                                   double* __restrict__ lmin, double* __restrict__ lmax) {
  const int blk = blockIdx.x * blockDim.x + threadIdx.x;
  if (blk >= nblk) return;
  // effective length: stop at a breakdown (beta ~ 0)
  int Ke = K;
  for (int j = 1; j < K; ++j)
    if (!(beta2[(size_t)j * nblk + blk] > 1e-24)) { Ke = j; break; }
  double lo = 1e300, hi = -1e300;
  for (int j = 0; j < Ke; ++j) {
    const double a = alpha[(size_t)j * nblk + blk];
    const double bl = j > 0 ? sqrt(beta2[(size_t)j * nblk + blk]) : 0.0;
    const double br = j + 1 < Ke ? sqrt(beta2[(size_t)(j + 1) * nblk + blk]) : 0.0;
    lo = fmin(lo, a - bl - br);
    hi = fmax(hi, a + bl + br);
  }
  // smallest: the least x with count(x) >= 1 ; largest: least x with count(x) >= Ke
  double l = lo, u = hi;
  for (int it = 0; it < 200 && u - l > 1e-13 * fmax(1.0, fabs(u) + fabs(l)); ++it) {
    const double m = 0.5 * (l + u);
    if (sturm_count(alpha, beta2, Ke, nblk, blk, m) >= 1) u = m; else l = m;
  }
  lmin[blk] = 0.5 * (l + u);
  l = lo; u = hi;
  for (int it = 0; it < 200 && u - l > 1e-13 * fmax(1.0, fabs(u) + fabs(l)); ++it) {
    const double m = 0.5 * (l + u);
    if (sturm_count(alpha, beta2, Ke, nblk, blk, m) >= Ke) u = m; else l = m;
  }
  lmax[blk] = 0.5 * (l + u);
}

// Replay of one Lanczos step with the scalars of the first pass (no reductions), accumulating the
// Ritz vector: y += s_j v ; t = w - alpha_j v - beta_j vprev ; vprev = v ; v = t / beta_{j+1}
template <typename R>
__global__ void k_lz_replay(const cplx<R>* __restrict__ w, cplx<R>* __restrict__ v, cplx<R>* __restrict__ vprev,
                            double2* __restrict__ y, int N, const double* __restrict__ s_j, const double* __restrict__ alpha,
                            const double* __restrict__ beta2, const double* __restrict__ beta2_next) {
  const int b = blockIdx.y;
  const double al = alpha[b];
  const double be = beta2 ? sqrt(fmax(beta2[b], 0.0)) : 0.0;
  const double bb = beta2_next[b];
  const double inv = bb > 1e-200 ? 1.0 / sqrt(bb) : 0.0;
  const double sj = s_j[b];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)b * N + i;
    const cplx<R> x = v[k], xp = vprev[k], ww = w[k];
    y[k].x += sj * (double)x.x;
    y[k].y += sj * (double)x.y;
    cplx<R> t;
    t.x = (R)((double)ww.x - al * x.x - be * xp.x);
    t.y = (R)((double)ww.y - al * x.y - be * xp.y);
    vprev[k] = x;
    t.x = (R)(t.x * inv);
    t.y = (R)(t.y * inv);
    v[k] = t;
  }
}
// Euclidean squared norm of each block's column of y (complex128)
__global__ void k_norm2_cols(const double2* __restrict__ y, int N, double* __restrict__ acc) {
  const int b = blockIdx.y;
  const double2* x = y + (size_t)b * N;
  double s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) s += x[i].x * x[i].x + x[i].y * x[i].y;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    atomicAdd(acc + b, t);
  }
}
__global__ void k_scale_cols(double2* __restrict__ y, int N, const double* __restrict__ n2) {
  const int b = blockIdx.y;
  const double inv = n2[b] > 0 ? 1.0 / sqrt(n2[b]) : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)b * N + i;
    y[k].x *= inv;
    y[k].y *= inv;
  }
}

// Effective Krylov length of block blk: the iteration stops at a breakdown (beta ~ 0); the same
// rule as k_tridiag_extremes.
static int lanczos_length(const std::vector<double>& beta2, int K, int nblk, int blk) {
  for (int j = 1; j < K; ++j)
    if (!(beta2[(size_t)j * nblk + blk] > 1e-24)) return j;
  return K;
}

// Eigenvector of the Ke x Ke Lanczos tridiagonal (diagonal alpha, squared off-diagonals beta2)
// for its eigenvalue mu, by inverse iteration with a dense pivoted solve (Ke <= 64).
static std::vector<double> tridiag_eigvec(const std::vector<double>& alpha, const std::vector<double>& beta2, int Ke, int nblk,
                                          int blk, double mu) {
  const double scale = std::max(1.0, std::fabs(mu));
  std::vector<double> x(Ke, 1.0), A((size_t)Ke * Ke);
  for (int it = 0; it < 4; ++it) {
    std::fill(A.begin(), A.end(), 0.0);
    for (int j = 0; j < Ke; ++j) {
      A[(size_t)j * Ke + j] = alpha[(size_t)j * nblk + blk] - mu;
      if (j > 0) {
        const double e = std::sqrt(std::max(0.0, beta2[(size_t)j * nblk + blk]));
        A[(size_t)j * Ke + j - 1] = e;
        A[(size_t)(j - 1) * Ke + j] = e;
      }
    }
    std::vector<double> b = x;
    // Gaussian elimination with partial pivoting (row-major A)
    for (int c = 0; c < Ke; ++c) {
      int p = c;
      for (int r = c + 1; r < Ke; ++r)
        if (std::fabs(A[(size_t)r * Ke + c]) > std::fabs(A[(size_t)p * Ke + c])) p = r;
      if (p != c) {
        for (int k = 0; k < Ke; ++k) std::swap(A[(size_t)p * Ke + k], A[(size_t)c * Ke + k]);
        std::swap(b[p], b[c]);
      }
      double piv = A[(size_t)c * Ke + c];
      if (std::fabs(piv) < 1e-14 * scale) piv = A[(size_t)c * Ke + c] = 1e-14 * scale;   // (near-)singular: the shift is an eigenvalue
      for (int r = c + 1; r < Ke; ++r) {
        const double f = A[(size_t)r * Ke + c] / piv;
        if (f == 0.0) continue;
        for (int k = c; k < Ke; ++k) A[(size_t)r * Ke + k] -= f * A[(size_t)c * Ke + k];
        b[r] -= f * b[c];
      }
    }
    for (int c = Ke - 1; c >= 0; --c) {
      double t = b[c];
      for (int k = c + 1; k < Ke; ++k) t -= A[(size_t)c * Ke + k] * x[k];
      x[c] = t / A[(size_t)c * Ke + c];
    }
    double n = 0;
    for (double v : x) n += v * v;
    n = std::sqrt(n);
    if (!(n > 0) || !std::isfinite(n)) { std::fill(x.begin(), x.end(), 0.0); x[0] = 1.0; break; }
    for (double& v : x) v /= n;
  }
  return x;
}

// Batched Lanczos over all blocks in the W inner product: fills lmin/lmax (host, nblk each).
// ubgv_in (host N x nblk complex128, may be null): start vector of each block whose column is
// not zero (the others start from the seeded random vector).  ubgv_out (may be null): the Ritz
// vector of the largest Ritz value of each block, 2-norm normalised, from a second pass that
// replays the recurrence with the first pass's scalars (no K x N vector storage).
template <typename R>
static cx_status lanczos_bounds(cx_handle h, int K, std::vector<double>& lmin, std::vector<double>& lmax, const double* ubgv_in,
                                double* ubgv_out) {
  const int nblk = h->nblk, N = h->g.N;
  const size_t vec = (size_t)N * nblk * sizeof(cplx<R>);
  const size_t yvec = ubgv_out ? (size_t)N * nblk * sizeof(double2) : 0;
  const int nseg = std::max(1, h->nl.nseg);
  const size_t cpb = (size_t)nblk * nseg * kAngMax * sizeof(cplx<R>);
  const size_t sc = (size_t)(2 * (K + 1) * nblk + 3 * nblk + K * nblk) * sizeof(double);
  const size_t need = 3 * vec + yvec + cpb + sc + nblk * sizeof(BlockDev<R>) + nblk * sizeof(int2) + sizeof(StepScalars) * nblk + 2048;
  cx_status s = ensure(h, &h->d_lz, &h->lz_bytes, need);
  if (s != CX_OK) return s;
  char* p = (char*)h->d_lz;
  cplx<R>* v = (cplx<R>*)p; p += vec;
  cplx<R>* w = (cplx<R>*)p; p += vec;
  cplx<R>* vprev = (cplx<R>*)p; p += vec;
  p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
  double2* y = (double2*)p; p += yvec;
  cplx<R>* cprime = (cplx<R>*)p; p += cpb;
  double* alpha = (double*)p; p += (size_t)(K + 1) * nblk * sizeof(double);
  double* beta2 = (double*)p; p += (size_t)(K + 1) * nblk * sizeof(double);
  double* dmin = (double*)p; p += nblk * sizeof(double);
  double* dmax = (double*)p; p += nblk * sizeof(double);
  double* n2 = (double*)p; p += nblk * sizeof(double);
  double* svec = (double*)p; p += (size_t)K * nblk * sizeof(double);
  p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
  BlockDev<R>* d_blk = (BlockDev<R>*)p; p += nblk * sizeof(BlockDev<R>);
  int2* d_tab = (int2*)p; p += nblk * sizeof(int2);
  StepScalars* d_sc = (StepScalars*)p;

  std::vector<cplx<R>*> p0(nblk), p1(nblk);
  std::vector<int> ids(nblk);
  std::vector<int2> tab(nblk);
  for (int b = 0; b < nblk; ++b) { p0[b] = v + (size_t)b * N; p1[b] = w + (size_t)b * N; ids[b] = b; tab[b] = make_int2(b, 0); }
  std::vector<BlockDev<R>> bd;
  make_block_devs<R>(h, p0, p1, ids, bd);
  for (auto& d : bd) d.Ns = 1;
  std::vector<StepScalars> one(nblk, StepScalars{1.0, 0.0, 0.0, 0.0});
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_blk, bd.data(), nblk * sizeof(BlockDev<R>), cudaMemcpyHostToDevice, h->stream));
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_tab, tab.data(), nblk * sizeof(int2), cudaMemcpyHostToDevice, h->stream));
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_sc, one.data(), nblk * sizeof(StepScalars), cudaMemcpyHostToDevice, h->stream));
  CX_TRY_CUDA(h, cudaMemsetAsync(alpha, 0, 2 * (K + 1) * nblk * sizeof(double), h->stream));

  const dim3 rg((unsigned)std::min(64, (N + 255) / 256), (unsigned)nblk);
  // start vectors: seeded random, replaced by the caller's guess where its column is not zero
  std::vector<char> guess(nblk, 0);
  if (ubgv_in)
    for (int b = 0; b < nblk; ++b) {
      const double* col = ubgv_in + 2 * (size_t)N * b;
      for (size_t i = 0; i < 2 * (size_t)N; ++i)
        if (col[i] != 0.0) { guess[b] = 1; break; }
    }
  auto start_vectors = [&]() -> cx_status {
    k_lz_init<R><<<grid_for((size_t)N * nblk), 256, 0, h->stream>>>(v, vprev, N, nblk, 12345u);
    h->launches++;
    for (int b = 0; b < nblk; ++b)
      if (guess[b]) {
        cx_status st = cx_host_to_dev(h, ubgv_in + 2 * (size_t)N * b, v + (size_t)b * N, N, sizeof(R) == 4 ? CX_PREC_MIXED : CX_PREC_FP64);
        if (st != CX_OK) return st;
      }
    // ||v0||_W^2, then normalise
    CX_TRY_CUDA(h, cudaMemsetAsync(n2, 0, nblk * sizeof(double), h->stream));
    k_lz_dot<R><<<rg, 256, 0, h->stream>>>(v, v, h->d_W, N, n2);
    k_lz_norm0<R><<<rg, 256, 0, h->stream>>>(v, N, n2);
    h->launches += 2;
    return CX_OK;
  };
  if ((s = start_vectors()) != CX_OK) return s;
  for (int j = 0; j < K; ++j) {
    // w = H v
    cx_status st = fused_step<R>(h, d_blk, d_sc, nblk, d_tab, nblk, 0, false, cprime, true, 0.0);
    if (st != CX_OK) return st;
    k_lz_dot<R><<<rg, 256, 0, h->stream>>>(v, w, h->d_W, N, alpha + (size_t)j * nblk);
    k_lz_update<R><<<rg, 256, 0, h->stream>>>(w, v, vprev, h->d_W, N, alpha + (size_t)j * nblk,
                                              j > 0 ? beta2 + (size_t)j * nblk : nullptr, beta2 + (size_t)(j + 1) * nblk);
    k_lz_shift<R><<<rg, 256, 0, h->stream>>>(w, v, vprev, N, beta2 + (size_t)(j + 1) * nblk);
    h->launches += 3;
  }
  CX_TRY_CUDA(h, cudaGetLastError());
  k_tridiag_extremes<<<(nblk + 63) / 64, 64, 0, h->stream>>>(alpha, beta2, K, nblk, dmin, dmax);
  h->launches++;
  lmin.resize(nblk);
  lmax.resize(nblk);
  CX_TRY_CUDA(h, cudaMemcpyAsync(lmin.data(), dmin, nblk * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CX_TRY_CUDA(h, cudaMemcpyAsync(lmax.data(), dmax, nblk * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  if (!ubgv_out) return CX_OK;

  // ---- Ritz vector of lmax: eigenvector s of the tridiagonal (host), then y = sum_j s_j v_j
  std::vector<double> ha((size_t)(K + 1) * nblk), hb((size_t)(K + 1) * nblk), hs((size_t)K * nblk, 0.0);
  CX_TRY_CUDA(h, cudaMemcpy(ha.data(), alpha, ha.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CX_TRY_CUDA(h, cudaMemcpy(hb.data(), beta2, hb.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int b = 0; b < nblk; ++b) {
    const int Ke = lanczos_length(hb, K, nblk, b);
    const std::vector<double> x = tridiag_eigvec(ha, hb, Ke, nblk, b, lmax[b]);
    for (int j = 0; j < Ke; ++j) hs[(size_t)j * nblk + b] = x[j];
  }
  CX_TRY_CUDA(h, cudaMemcpyAsync(svec, hs.data(), hs.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CX_TRY_CUDA(h, cudaMemsetAsync(y, 0, yvec, h->stream));
  if ((s = start_vectors()) != CX_OK) return s;
  for (int j = 0; j < K; ++j) {
    cx_status st = fused_step<R>(h, d_blk, d_sc, nblk, d_tab, nblk, 0, false, cprime, true, 0.0);
    if (st != CX_OK) return st;
    k_lz_replay<R><<<rg, 256, 0, h->stream>>>(w, v, vprev, y, N, svec + (size_t)j * nblk, alpha + (size_t)j * nblk,
                                              j > 0 ? beta2 + (size_t)j * nblk : nullptr, beta2 + (size_t)(j + 1) * nblk);
    h->launches++;
  }
  CX_TRY_CUDA(h, cudaMemsetAsync(n2, 0, nblk * sizeof(double), h->stream));
  k_norm2_cols<<<rg, 256, 0, h->stream>>>(y, N, n2);
  k_scale_cols<<<rg, 256, 0, h->stream>>>(y, N, n2);
  h->launches += 2;
  CX_TRY_CUDA(h, cudaGetLastError());
  CX_TRY_CUDA(h, cudaMemcpyAsync(ubgv_out, y, yvec, cudaMemcpyDeviceToHost, h->stream));
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  return CX_OK;
}

// ------------------------------------------------------------------ Rayleigh-Ritz of one block
#define CX_TRY_BLAS(h, expr)                                                          \
  do {                                                                                \
    cublasStatus_t _s = (expr);                                                       \
    if (_s != CUBLAS_STATUS_SUCCESS) {                                                \
      (h)->err = std::string(#expr) + ": cuBLAS status " + std::to_string((int)_s);   \
      return CX_ERR_LIB;                                                              \
    }                                                                                 \
  } while (0)
#define CX_TRY_SOLVER(h, expr)                                                        \
  do {                                                                                \
    cusolverStatus_t _s = (expr);                                                     \
    if (_s != CUSOLVER_STATUS_SUCCESS) {                                              \
      (h)->err = std::string(#expr) + ": cuSOLVER status " + std::to_string((int)_s); \
      return CX_ERR_LIB;                                                              \
    }                                                                                 \
  } while (0)

constexpr int kRestarts = 4;      // similarity restarts of a stalled refinement before the general solver
constexpr int kRestartGiveUp = 4; // blocks in a row that needed the general solver after restarts: stop
                                  // restarting for the rest of the eigSolver call
constexpr int kGeevMax = 512;     // largest block for the general FP64 solver (about 1 s at n = 1000)
constexpr double kRotMinDiag = 1e-3;   // smallest Cholesky diagonal of the rotated block's unit-diagonal W-Gram

struct RRWork {
  double2 *G, *Hs, *V, *ev;
  double2 *Gw, *T, *U, *B, *Z, *Zn, *EZ, *Hs0;   // subspace eigensolver (W-similarity + refinement)
  double *wh, *dmax;
  float2 *Gf, *Mf, *Cf;
  double* scfac;
  int* perm;
  int* info;
  double2* Zbest;            // best iterate of a stalled refinement (restart point)
  int64_t* ipiv;             // LU pivots of a restart
  double2* T0;               // the W-similar matrix T, kept for the Hermitian-part eigenpairs
  double* rmin;              // smallest Cholesky diagonal of the rotation check
  float* img;                // the rotation coefficients in the tensor-core operand layout
};

static cx_status rr_workspace(cx_handle h, int nmax, int ncolmax, RRWork& w) {
  const size_t n2 = (size_t)nmax * nmax;
  const size_t need = n2 * 16 * 13 + nmax * 16 + nmax * 8 + 64 + n2 * 8 * 3 + (size_t)ncolmax * 8 + nmax * 4 + 64 + nmax * 8 + 64 +
                      tc_rot_image_floats(nmax, nmax) * 4 + 48 * 256;
  cx_status s = ensure(h, &h->d_rr, &h->rr_bytes, need);
  if (s != CX_OK) return s;
  char* p = (char*)h->d_rr;
  auto take = [&](size_t bytes) { char* q = p; p += (bytes + 255) & ~(size_t)255; return (void*)q; };
  w.G = (double2*)take(n2 * 16);
  w.Hs = (double2*)take(n2 * 16);
  w.V = (double2*)take(n2 * 16);
  w.ev = (double2*)take(nmax * 16);
  w.Gw = (double2*)take(n2 * 16);
  w.T = (double2*)take(n2 * 16);
  w.U = (double2*)take(n2 * 16);
  w.B = (double2*)take(n2 * 16);
  w.Z = (double2*)take(n2 * 16);
  w.Zn = (double2*)take(n2 * 16);
  w.EZ = (double2*)take(n2 * 16);
  w.Hs0 = (double2*)take(n2 * 16);
  w.wh = (double*)take(nmax * 8);
  w.dmax = (double*)take(64);
  w.Gf = (float2*)take(n2 * 8);
  w.Mf = (float2*)take(n2 * 8);
  w.Cf = (float2*)take(n2 * 8);
  w.scfac = (double*)take((size_t)ncolmax * 8);
  w.perm = (int*)take(nmax * 4);
  w.info = (int*)take(64);
  w.Zbest = (double2*)take(n2 * 16);
  w.ipiv = (int64_t*)take((size_t)nmax * 8);
  w.T0 = (double2*)take(n2 * 16);
  w.rmin = (double*)take(64);
  w.img = (float*)take(tc_rot_image_floats(nmax, nmax) * 4);
  return CX_OK;
}

// Gram and projected matrices into w.G (X^H X) and w.Hs (X^H HX), complex128.
template <typename R>
static cx_status rr_gemms(cx_handle h, const cplx<R>* X, const cplx<R>* HX, int N, int n, RRWork& w);

template <>
cx_status rr_gemms<double>(cx_handle h, const double2* X, const double2* HX, int N, int n, RRWork& w) {
  const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
  CX_TRY_BLAS(h, cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
  CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, N, &one, (const cuDoubleComplex*)X, N,
                             (const cuDoubleComplex*)X, N, &zero, (cuDoubleComplex*)w.G, n));
  CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, N, &one, (const cuDoubleComplex*)X, N,
                             (const cuDoubleComplex*)HX, N, &zero, (cuDoubleComplex*)w.Hs, n));
  return CX_OK;
}

template <>
cx_status rr_gemms<float>(cx_handle h, const float2* X, const float2* HX, int N, int n, RRWork& w) {
  // Gram and projected matrices on the tensor cores (3xTF32 products, FP32 accumulation over short
  // ranges, FP64 sums)
  cx_status s = tc_gram(h, X, X, nullptr, N, n, n, w.G, n);
  if (s != CX_OK) return s;
  return tc_gram(h, X, HX, nullptr, N, n, n, w.Hs, n);
}

// Gw = X^H Y (complex128)
static cx_status rr_gram(cx_handle h, const double2* X, const double2* Y, int N, int n, RRWork& w) {
  const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
  CX_TRY_BLAS(h, cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
  CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, N, &one, (const cuDoubleComplex*)X, N, (const cuDoubleComplex*)Y,
                             N, &zero, (cuDoubleComplex*)w.Gw, n));
  return CX_OK;
}
// Gw = X^H W X for complex64 X: the weights are applied on the tensor-core operand load
static cx_status rr_wgram(cx_handle h, const float2* X, int N, int n, RRWork& w) {
  return tc_gram(h, X, X, h->d_W32, N, n, n, w.Gw, n);
}

template <typename R>
static cx_status rr_rotate(cx_handle h, const cplx<R>* X, cplx<R>* out, int N, int n, RRWork& w);

template <>
cx_status rr_rotate<double>(cx_handle h, const double2* X, double2* out, int N, int n, RRWork& w) {
  const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
  CX_TRY_BLAS(h, cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
  CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, N, n, n, &one, (const cuDoubleComplex*)X, N,
                             (const cuDoubleComplex*)w.V, n, &zero, (cuDoubleComplex*)out, N));
  return CX_OK;
}

template <>
cx_status rr_rotate<float>(cx_handle h, const float2* X, float2* out, int N, int n, RRWork& w) {
  return tc_rotate(h, X, w.V, N, n, n, out, w.img);
}

// Eigenpairs of the Ritz pencil A = G^-1 M (w.Hs, n x n complex128, not Hermitian for Cyclix
// cells) into w.ev and the rotation coefficients c into w.V.  With the W-Gram Gw = X^H W X =
// U_w^H U_w, T = U_w A U_w^-1 is similar to A and Hermitian up to the subspace residual (the
// Hamiltonian is self-adjoint in the W inner product).  Tier 1 iterates the fixed point
// T X = X Lambda with X = I + Z directly; tier 2 starts it from the Hermitian eigenvectors U of
// (T + T^H)/2 (B = U^H T U); c = U_w^-1 (U) X.  When neither converges (clustered spectrum, first
// steps) the general solver cusolverDnXgeev runs on Hs = R A R^-1 (R = chol(G) in w.G) and
// c = R^-1 v, for blocks of at most kGeevMax states.
// Every result must leave the rotated block well conditioned: the W-Gram of X c is Y^H Y with
// Y = U_w c (the eigenvectors of T), and its unit-diagonal Cholesky factor must keep every
// diagonal entry above kRotMinDiag.  A fixed point can converge to a degenerate solution (several
// columns on one eigenvector) and a non-normal T can give nearly parallel general eigenvectors;
// either is rejected.  The last resort is the Hermitian part itself: eigenvalues and eigenvectors
// of (T + T^H)/2, whose real eigenvalues differ from the real parts of T's eigenvalues only at
// second order in the anti-Hermitian part (its first-order term u^H T_a u is imaginary), with a
// W-orthonormal rotation.  *path: 0 refinement, 1 general solver, 2 Hermitian part.
static cx_status subspace_eig(cx_handle h, int n, RRWork& w, int* path, int* tier) {
  const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
  const size_t n2 = (size_t)n * n;
  const unsigned gn = grid_for(n2);
  cudaStream_t st = h->stream;
  *path = 0;
  CX_TRY_BLAS(h, cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
  CX_TRY_CUDA(h, cudaMemcpyAsync(w.Hs0, w.Hs, n2 * 16, cudaMemcpyDeviceToDevice, st));
  // U_w = chol(Gw) (upper)
  size_t wsd = 0, wsh = 0;
  CX_TRY_SOLVER(h, cusolverDnXpotrf_bufferSize(h->cusolver, h->cusolver_params, CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, w.Gw, n,
                                                CUDA_C_64F, &wsd, &wsh));
  size_t wsd2 = 0, wsh2 = 0;
  CX_TRY_SOLVER(h, cusolverDnXsyevd_bufferSize(h->cusolver, h->cusolver_params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                                CUDA_C_64F, w.U, n, CUDA_R_64F, w.wh, CUDA_C_64F, &wsd2, &wsh2));
  wsd = std::max(wsd, wsd2);
  wsh = std::max(wsh, wsh2);
  const bool mixed = h->prec == CX_PREC_MIXED;
  if (mixed) {
    CX_TRY_SOLVER(h, cusolverDnXsyevd_bufferSize(h->cusolver, h->cusolver_params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                                  CUDA_C_32F, w.Mf, n, CUDA_R_32F, w.Cf, CUDA_C_32F, &wsd2, &wsh2));
    wsd = std::max(wsd, wsd2);
    wsh = std::max(wsh, wsh2);
  }
  cx_status s;
  if ((s = ensure(h, &h->d_ws, &h->ws_bytes, wsd + 256)) != CX_OK) return s;
  if (h->hws_bytes < wsh + 256) {
    cudaFreeHost(h->h_ws);
    h->h_ws = nullptr;
    h->hws_bytes = 0;
    CX_TRY_CUDA(h, cudaMallocHost(&h->h_ws, wsh + 256));
    h->hws_bytes = wsh + 256;
  }
  CX_TRY_SOLVER(h, cusolverDnXpotrf(h->cusolver, h->cusolver_params, CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, w.Gw, n, CUDA_C_64F,
                                     h->d_ws, h->ws_bytes, h->h_ws, h->hws_bytes, w.info));
  int info = 0;
  CX_TRY_CUDA(h, cudaMemcpyAsync(&info, w.info, sizeof(int), cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  bool fast = info == 0;
  // is the block X c, c in w.V, well conditioned in the W inner product?  (w.EZ, w.B are scratch)
  auto rotation_ok = [&](bool* ok) -> cx_status {
    *ok = false;
    CX_TRY_BLAS(h, cublasZtrmm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                               (const cuDoubleComplex*)w.Gw, n, (const cuDoubleComplex*)w.V, n, (cuDoubleComplex*)w.EZ, n));
    CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.EZ, n,
                               (const cuDoubleComplex*)w.EZ, n, &zero, (cuDoubleComplex*)w.B, n));
    k_unit_diag<<<gn, 256, 0, st>>>(w.B, n);
    k_unit_diag_fix<<<(n + 255) / 256, 256, 0, st>>>(w.B, n);
    h->launches += 2;
    CX_TRY_SOLVER(h, cusolverDnXpotrf(h->cusolver, h->cusolver_params, CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, w.B, n, CUDA_C_64F,
                                       h->d_ws, h->ws_bytes, h->h_ws, h->hws_bytes, w.info));
    k_min_diag<<<1, 256, 0, st>>>(w.B, n, w.rmin);
    h->launches++;
    int inf = 0;
    double rmin = 0;
    CX_TRY_CUDA(h, cudaMemcpyAsync(&inf, w.info, sizeof(int), cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaMemcpyAsync(&rmin, w.rmin, sizeof(double), cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    *ok = inf == 0 && rmin > kRotMinDiag;
    return CX_OK;
  };
  // The refined eigenvectors X = I + Z (in w.Z) of a nearly diagonal matrix: when ||Z||_F <= 1/2,
  // the rotated block's W-Gram (I + Z)^H (I + Z) (times a unitary U in tier 2) has its smallest
  // unit-diagonal Cholesky diagonal above 1/3 > kRotMinDiag, so the check can be skipped.
  auto near_identity = [&](bool* yes) -> cx_status {
    k_dist_identity2<<<1, 512, 0, st>>>(w.Z, n, w.rmin);
    h->launches++;
    double d2 = 1e300;
    CX_TRY_CUDA(h, cudaMemcpyAsync(&d2, w.rmin, sizeof(double), cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    *yes = d2 <= 0.25;
    return CX_OK;
  };
  bool have_herm = false;     // w.U / w.wh hold the eigenpairs of (T + T^H)/2
  bool herm_fp32 = false;     // ... computed in FP32 (the mixed path's starting point of tier 2)
  // In the mixed path tier 2 starts from FP32 eigenvectors (cheevd: at GB300's FP64 rate the FP64
  // tridiagonalisation was the costliest step of the Rayleigh-Ritz), which its FP64 refinement of
  // B = U^H T U corrects; full: FP64 eigenpairs (the Hermitian-part result and large blocks).
  auto hermitian_eig = [&](bool full) -> cx_status {
    k_herm_part<<<gn, 256, 0, st>>>(w.T0, w.U, n);
    h->launches++;
    herm_fp32 = mixed && !full;
    if (herm_fp32) {
      k_d2f<<<gn, 256, 0, st>>>(w.U, w.Mf, n2);
      CX_TRY_SOLVER(h, cusolverDnXsyevd(h->cusolver, h->cusolver_params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_32F,
                                         w.Mf, n, CUDA_R_32F, w.Cf, CUDA_C_32F, h->d_ws, h->ws_bytes, h->h_ws, h->hws_bytes, w.info));
      k_f2d<<<gn, 256, 0, st>>>(w.Mf, w.U, n2);
      k_r2d<<<(n + 255) / 256, 256, 0, st>>>((const float*)w.Cf, w.wh, n);
      h->launches += 3;
    } else {
      CX_TRY_SOLVER(h, cusolverDnXsyevd(h->cusolver, h->cusolver_params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_64F,
                                         w.U, n, CUDA_R_64F, w.wh, CUDA_C_64F, h->d_ws, h->ws_bytes, h->h_ws, h->hws_bytes, w.info));
    }
    CX_TRY_CUDA(h, cudaMemcpyAsync(&info, w.info, sizeof(int), cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    if (info != 0) {
      h->err = "eigensolver: Hermitian eigensolver failed (info " + std::to_string(info) + ")";
      return CX_ERR_LIB;
    }
    have_herm = true;
    return CX_OK;
  };
  // fixed-point refinement of B X = X Lambda (B in w.B is split in place into diag -> w.ev, off-diag);
  // returns true when converged, with lambda in w.ev and X = I + Z in w.Z
  // The mixed path runs the first sweeps with the B Z product on the tensor cores (complex64
  // operands, FP32-accurate BF16x9 products) down to the FP32 level, then finishes in complex128.
  double best_dm = 1e300;   // best step size of the last refine() call; its iterate is in w.Zbest
  auto refine = [&](bool* conv) -> cx_status {
    *conv = false;
    best_dm = 1e300;
    k_split_diag<<<gn, 256, 0, st>>>(w.B, w.ev, w.Z, n);
    h->launches++;
    bool fp32 = mixed;
    if (fp32) {
      k_d2f<<<gn, 256, 0, st>>>(w.B, w.Gf, n2);
      h->launches++;
    }
    double prev = 1e300;
    for (int it = 0; it < 80; ++it) {
      CX_TRY_CUDA(h, cudaMemsetAsync(w.dmax, 0, 8, st));
      if (fp32) {
        const cuComplex c1 = make_cuComplex(1, 0), c0 = make_cuComplex(0, 0);
        k_d2f<<<gn, 256, 0, st>>>(w.Z, w.Mf, n2);
        CX_TRY_BLAS(h, cublasSetMathMode(h->cublas, CUBLAS_FP32_EMULATED_BF16X9_MATH));
        CX_TRY_BLAS(h, cublasCgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &c1, (const cuComplex*)w.Gf, n,
                                   (const cuComplex*)w.Mf, n, &c0, (cuComplex*)w.Cf, n));
        CX_TRY_BLAS(h, cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
        k_sylv_update<float2><<<gn, 256, 0, st>>>(w.B, w.Cf, w.ev, w.Z, w.Zn, n, (unsigned long long*)w.dmax);
        h->launches += 2;
      } else {
        CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.B, n,
                                   (const cuDoubleComplex*)w.Z, n, &zero, (cuDoubleComplex*)w.EZ, n));
        k_sylv_update<double2><<<gn, 256, 0, st>>>(w.B, w.EZ, w.ev, w.Z, w.Zn, n, (unsigned long long*)w.dmax);
        h->launches++;
      }
      std::swap(w.Z, w.Zn);
      double dm = 0;
      CX_TRY_CUDA(h, cudaMemcpyAsync(&dm, w.dmax, 8, cudaMemcpyDeviceToHost, st));
      CX_TRY_CUDA(h, cudaStreamSynchronize(st));
      if (!(dm < 1e300)) return CX_OK;                       // diverged (inf / NaN)
      if (dm < best_dm) {
        best_dm = dm;
        CX_TRY_CUDA(h, cudaMemcpyAsync(w.Zbest, w.Z, n2 * 16, cudaMemcpyDeviceToDevice, st));
      }
      if (fp32) {
        // FP32 level reached (or the complex64 sweeps stall): continue in complex128
        if (dm < 1e-6 || (it >= 8 && dm > 0.9 * prev)) { fp32 = false; prev = 1e300; }
        else prev = dm;
        continue;
      }
      // (the mixed path's Hs carries FP32-level errors: polishing below 1e-8 changes nothing)
      if (dm < (mixed ? 1e-8 : 1e-12)) { *conv = true; break; }
      if (it >= 8 && dm > 0.9 * prev) return CX_OK;          // not contracting
      prev = dm;
    }
    if (!*conv) return CX_OK;
    CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.B, n,
                               (const cuDoubleComplex*)w.Z, n, &zero, (cuDoubleComplex*)w.EZ, n));
    k_sylv_finish<<<gn, 256, 0, st>>>(w.EZ, w.ev, w.Z, w.ev, n);
    h->launches++;
    return CX_OK;
  };
  if (fast) {
    // T = (U_w A) U_w^-1
    CX_TRY_BLAS(h, cublasZtrmm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                               (const cuDoubleComplex*)w.Gw, n, (const cuDoubleComplex*)w.Hs, n, (cuDoubleComplex*)w.T, n));
    CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                               (const cuDoubleComplex*)w.Gw, n, (cuDoubleComplex*)w.T, n));
    CX_TRY_CUDA(h, cudaMemcpyAsync(w.T0, w.T, n2 * 16, cudaMemcpyDeviceToDevice, st));
    // tier 1: the filtered block is ordered like the previous Ritz vectors, so near self-consistency T
    // itself is nearly diagonal -- refine directly (U = I).  Skipped when this block needed tier 2
    // in its previous step (degenerate clusters keep the fixed point from converging).
    bool conv = false;
    cx_status rs = CX_OK;
    const bool try_tier1 = *tier != 2;
    *tier = 2;
    if (try_tier1) {
      CX_TRY_CUDA(h, cudaMemcpyAsync(w.B, w.T, n2 * 16, cudaMemcpyDeviceToDevice, st));
      rs = refine(&conv);
      if (rs != CX_OK) return rs;
    }
    if (conv) {
      // eigenvectors of A: c = U_w^-1 X
      bool ok = false;
      if ((rs = near_identity(&ok)) != CX_OK) return rs;
      CX_TRY_CUDA(h, cudaMemcpyAsync(w.V, w.Z, n2 * 16, cudaMemcpyDeviceToDevice, st));
      CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                                 (const cuDoubleComplex*)w.Gw, n, (cuDoubleComplex*)w.V, n));
      if (!ok && (rs = rotation_ok(&ok)) != CX_OK) return rs;
      if (ok) {
        *tier = 1;
        return CX_OK;
      }
    }
    // tier 2: Hermitian eigenvectors U of (T + T^H)/2, then refine B = U^H T U (blocks of more than
    // kGeevMax states go to the Hermitian part directly: their refinement does not converge while
    // the top of the block is unconverged, and its sweeps cost O(n^3) each)
    if ((rs = hermitian_eig(n > kGeevMax)) != CX_OK) return rs;
    if (n > kGeevMax) goto hermitian_part;
    CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.T0, n,
                               (const cuDoubleComplex*)w.U, n, &zero, (cuDoubleComplex*)w.EZ, n));
    CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.U, n,
                               (const cuDoubleComplex*)w.EZ, n, &zero, (cuDoubleComplex*)w.B, n));
    {
      // B X = X Lambda by the fixed point; when it stalls, restart from the similar matrix
      // X^-1 B X with X = I + Z of the best iterate (each restart shrinks the coupling
      // quadratically), accumulating the transforms in Xt (w.V, starting at U).  Bfull (w.T)
      // keeps the matrix of the current round, since refine() splits w.B.
      CX_TRY_CUDA(h, cudaMemcpyAsync(w.T, w.B, n2 * 16, cudaMemcpyDeviceToDevice, st));
      CX_TRY_CUDA(h, cudaMemcpyAsync(w.V, w.U, n2 * 16, cudaMemcpyDeviceToDevice, st));
      const int max_round = h->restart_fail_streak >= kRestartGiveUp ? 0 : kRestarts;
      for (int round = 0; round <= max_round; ++round) {
        if (round > 0) CX_TRY_CUDA(h, cudaMemcpyAsync(w.B, w.T, n2 * 16, cudaMemcpyDeviceToDevice, st));
        if ((rs = refine(&conv)) != CX_OK) return rs;
        if (conv) {
          // eigenvectors of A: c = U_w^-1 (Xt X); on the first round Xt = U is unitary
          bool ok = false;
          if (round == 0 && (rs = near_identity(&ok)) != CX_OK) return rs;
          CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.V, n,
                                     (const cuDoubleComplex*)w.Z, n, &zero, (cuDoubleComplex*)w.Hs, n));
          CX_TRY_CUDA(h, cudaMemcpyAsync(w.V, w.Hs, n2 * 16, cudaMemcpyDeviceToDevice, st));
          CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n,
                                     &one, (const cuDoubleComplex*)w.Gw, n, (cuDoubleComplex*)w.V, n));
          if (!ok && (rs = rotation_ok(&ok)) != CX_OK) return rs;
          if (ok) {
            h->eig_restarts += round;
            if (round > 0) h->restart_fail_streak = 0;
            return CX_OK;
          }
          break;                                                // degenerate fixed point
        }
        if (round == max_round || !(best_dm < 1.0)) {
          if (round > 0) h->restart_fail_streak++;
          break;
        }
        // X = I + Z_best;  Bfull <- X^-1 (Bfull X);  Xt <- Xt X
        k_add_identity<<<gn, 256, 0, st>>>(w.Zbest, n);
        h->launches++;
        CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.T, n,
                                   (const cuDoubleComplex*)w.Zbest, n, &zero, (cuDoubleComplex*)w.Hs, n));
        CX_TRY_CUDA(h, cudaMemcpyAsync(w.EZ, w.Zbest, n2 * 16, cudaMemcpyDeviceToDevice, st));
        size_t lwd = 0, lwh = 0;
        CX_TRY_SOLVER(h, cusolverDnXgetrf_bufferSize(h->cusolver, h->cusolver_params, n, n, CUDA_C_64F, w.EZ, n, CUDA_C_64F, &lwd,
                                                      &lwh));
        if ((s = ensure(h, &h->d_ws, &h->ws_bytes, lwd + 256)) != CX_OK) return s;
        if (h->hws_bytes < lwh + 256) {
          cudaFreeHost(h->h_ws);
          h->h_ws = nullptr;
          h->hws_bytes = 0;
          CX_TRY_CUDA(h, cudaMallocHost(&h->h_ws, lwh + 256));
          h->hws_bytes = lwh + 256;
        }
        CX_TRY_SOLVER(h, cusolverDnXgetrf(h->cusolver, h->cusolver_params, n, n, CUDA_C_64F, w.EZ, n, w.ipiv, CUDA_C_64F, h->d_ws,
                                           h->ws_bytes, h->h_ws, h->hws_bytes, w.info));
        CX_TRY_SOLVER(h, cusolverDnXgetrs(h->cusolver, h->cusolver_params, CUBLAS_OP_N, n, n, CUDA_C_64F, w.EZ, n, w.ipiv, CUDA_C_64F,
                                           w.Hs, n, w.info));
        CX_TRY_CUDA(h, cudaMemcpyAsync(&info, w.info, sizeof(int), cudaMemcpyDeviceToHost, st));
        CX_TRY_CUDA(h, cudaStreamSynchronize(st));
        if (info != 0) {                                        // singular transform: general solver
          h->restart_fail_streak++;
          break;
        }
        CX_TRY_CUDA(h, cudaMemcpyAsync(w.T, w.Hs, n2 * 16, cudaMemcpyDeviceToDevice, st));
        CX_TRY_BLAS(h, cublasZgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, (const cuDoubleComplex*)w.V, n,
                                   (const cuDoubleComplex*)w.Zbest, n, &zero, (cuDoubleComplex*)w.Hs, n));
        CX_TRY_CUDA(h, cudaMemcpyAsync(w.V, w.Hs, n2 * 16, cudaMemcpyDeviceToDevice, st));
      }
    }
  }
  if (!fast || n <= kGeevMax) {
    // general FP64 eigensolver on Hs = R A R^-1 (the reference's matrix, better conditioned than A)
    *path = 1;
    CX_TRY_BLAS(h, cublasZtrmm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                               (const cuDoubleComplex*)w.G, n, (const cuDoubleComplex*)w.Hs0, n, (cuDoubleComplex*)w.Hs, n));
    CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                               (const cuDoubleComplex*)w.G, n, (cuDoubleComplex*)w.Hs, n));
    size_t g1 = 0, g2 = 0;
    CX_TRY_SOLVER(h, cusolverDnXgeev_bufferSize(h->cusolver, h->cusolver_params, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_VECTOR, n,
                                                 CUDA_C_64F, w.Hs, n, CUDA_C_64F, w.ev, CUDA_C_64F, nullptr, n, CUDA_C_64F, w.V, n,
                                                 CUDA_C_64F, &g1, &g2));
    if ((s = ensure(h, &h->d_ws, &h->ws_bytes, g1 + 256)) != CX_OK) return s;
    if (h->hws_bytes < g2 + 256) {
      cudaFreeHost(h->h_ws);
      h->h_ws = nullptr;
      h->hws_bytes = 0;
      CX_TRY_CUDA(h, cudaMallocHost(&h->h_ws, g2 + 256));
      h->hws_bytes = g2 + 256;
    }
    CX_TRY_SOLVER(h, cusolverDnXgeev(h->cusolver, h->cusolver_params, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_VECTOR, n,
                                      CUDA_C_64F, w.Hs, n, CUDA_C_64F, w.ev, CUDA_C_64F, nullptr, n, CUDA_C_64F, w.V, n, CUDA_C_64F,
                                      h->d_ws, h->ws_bytes, h->h_ws, h->hws_bytes, w.info));
    CX_TRY_CUDA(h, cudaMemcpyAsync(&info, w.info, sizeof(int), cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    if (info != 0) {
      h->err = "eigensolver: geev failed (info " + std::to_string(info) + ")";
      return CX_ERR_LIB;
    }
    // rotation coefficients c = R^-1 v
    CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                               (const cuDoubleComplex*)w.G, n, (cuDoubleComplex*)w.V, n));
    if (!fast) return CX_OK;                                   // (no W-Cholesky factor to check against)
    bool ok = false;
    cx_status rs = rotation_ok(&ok);
    if (rs != CX_OK) return rs;
    if (ok) return CX_OK;
  }
  // Hermitian part: eigenvalues wh (real), c = U_w^-1 U
hermitian_part:
  *path = 2;
  if (!have_herm || herm_fp32) {
    // the final rotation: FP64 eigenpairs (FP32 vectors here slowed the 384-atom SCF's convergence
    // from a 2e-6 to a 1e-5 floor)
    cx_status rs = hermitian_eig(true);
    if (rs != CX_OK) return rs;
  }
  k_real_to_complex<<<(n + 255) / 256, 256, 0, st>>>(w.wh, w.ev, n);
  h->launches++;
  CX_TRY_CUDA(h, cudaMemcpyAsync(w.V, w.U, n2 * 16, cudaMemcpyDeviceToDevice, st));
  CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                             (const cuDoubleComplex*)w.Gw, n, (cuDoubleComplex*)w.V, n));
  return CX_OK;
}

template <typename R>
static cx_status rayleigh_ritz_block(cx_handle h, int b, int sel, RRWork& w, double* eig_out) {
  const int N = h->g.N, n = h->blocks[b].Ns;
  const cplx<R>* X = (const cplx<R>*)h->bufs[2 * b + sel];
  cplx<R>* HX = (cplx<R>*)h->bufs[2 * b + (sel ^ 1)];
  cx_status s = rr_gemms<R>(h, X, HX, N, n, w);
  if (s != CX_OK) return s;
  // W-weighted Gram (needed by the subspace eigensolver): Gw = X^H (W X)
  if constexpr (sizeof(R) == 4) {
    if ((s = rr_wgram(h, X, N, n, w)) != CX_OK) return s;
  } else {
    // complex128: W X in the H X buffer, then ZGEMM
    k_wscale<R><<<col_grid(N, n), 256, 0, h->stream>>>(X, HX, h->d_W, N, n);
    h->launches++;
    if ((s = rr_gram(h, X, HX, N, n, w)) != CX_OK) return s;
  }
  // Cholesky G = R^H R (upper)
  size_t wsd = 0, wsh = 0;
  CX_TRY_SOLVER(h, cusolverDnXpotrf_bufferSize(h->cusolver, h->cusolver_params, CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, w.G, n,
                                                CUDA_C_64F, &wsd, &wsh));
  if ((s = ensure(h, &h->d_ws, &h->ws_bytes, wsd + 256)) != CX_OK) return s;
  if (h->hws_bytes < wsh + 256) {
    cudaFreeHost(h->h_ws);
    h->h_ws = nullptr;
    h->hws_bytes = 0;
    CX_TRY_CUDA(h, cudaMallocHost(&h->h_ws, wsh + 256));
    h->hws_bytes = wsh + 256;
  }
  CX_TRY_SOLVER(h, cusolverDnXpotrf(h->cusolver, h->cusolver_params, CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, w.G, n, CUDA_C_64F,
                                     h->d_ws, h->ws_bytes, h->h_ws, h->hws_bytes, w.info));
  int info = 0;
  CX_TRY_CUDA(h, cudaMemcpyAsync(&info, w.info, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  if (info != 0) {
    h->err = "eigensolver: Gram matrix of block " + std::to_string(b) + " not positive definite (potrf info " + std::to_string(info) +
             "): the filtered block lost rank";
    return CX_ERR_NOTPD;
  }
  const cuDoubleComplex one = make_cuDoubleComplex(1, 0);
  CX_TRY_BLAS(h, cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
  // A = G^-1 M = R^-1 R^-H M: the Ritz pencil M c = lambda G c.  The reference's projected matrix
  // in the orthonormal basis Q = X R^-1 (the span of orth(X)) is Hs = R A R^-1, with the same
  // eigenvalues; its eigenvectors map to the rotation coefficients c = R^-1 v.
  CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                             (const cuDoubleComplex*)w.G, n, (cuDoubleComplex*)w.Hs, n));
  CX_TRY_BLAS(h, cublasZtrsm(h->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                             (const cuDoubleComplex*)w.G, n, (cuDoubleComplex*)w.Hs, n));
  // eigenpairs of Hs (general; eigSolver.m:110 -- Hs is not Hermitian for Cyclix cells)
  int path = 0;
  int tier_scratch = 0;
  int* tier = (h->rr_tier && b < h->rr_tier_n) ? &h->rr_tier[b] : &tier_scratch;
  if ((s = subspace_eig(h, n, w, &path, tier)) != CX_OK) return s;
  h->eig_fallbacks += path == 1 ? 1 : 0;
  h->eig_hermitian += path == 2 ? 1 : 0;
  std::vector<std::complex<double>> ev(n);
  CX_TRY_CUDA(h, cudaMemcpyAsync(ev.data(), w.ev, n * 16, cudaMemcpyDeviceToHost, h->stream));
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  // real part, ascending sort (eigSolver.m:111-116)
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int c) { return ev[a].real() < ev[c].real(); });
  for (int j = 0; j < n; ++j) eig_out[j] = ev[perm[j]].real();
  CX_TRY_CUDA(h, cudaMemcpyAsync(w.perm, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  k_gather_cols<<<grid_for((size_t)n * n), 256, 0, h->stream>>>(w.V, w.Hs, n, w.perm);
  h->launches++;
  // rotation coefficients C (sorted eigenvectors of the pencil, into w.V)
  CX_TRY_CUDA(h, cudaMemcpyAsync(w.V, w.Hs, (size_t)n * n * 16, cudaMemcpyDeviceToDevice, h->stream));
  // psi = X C  (into the other buffer), then W-normalise (eigSolver.m:119-124)
  if ((s = rr_rotate<R>(h, X, HX, N, n, w)) != CX_OK) return s;
  if constexpr (sizeof(R) == 4) {
    if ((s = check_pipeline_status(h)) != CX_OK) return s;
  }
  k_colnorm_w<R><<<n, 256, 0, h->stream>>>(HX, (const typename WOf<R>::T*)(sizeof(R) == 4 ? (const void*)h->d_W32 : (const void*)h->d_W), N,
                                          w.scfac);
  k_colscale<R><<<col_grid(N, n), 256, 0, h->stream>>>(HX, N, n, w.scfac);
  h->launches += 2;
  CX_TRY_CUDA(h, cudaGetLastError());
  return CX_OK;
}

// The Rayleigh-Ritz steps of all blocks.  Each block's step is a chain of small dependent
// operations (Gram products, Cholesky, the subspace eigensolver with its convergence tests on the
// host), so the blocks run concurrently: up to kRRWorkers host threads, each with its own stream,
// cuBLAS / cuSOLVER handles and workspace (a copy of the handle that points at them), take the
// blocks in turn.  The workers start after the filtered block and H X are complete on the handle's
// stream, and the handle continues after every worker has finished.
constexpr int kRRWorkers = 8;

static cx_status make_worker(cx_handle h, cx_rr_worker& wk) {
  CX_TRY_CUDA(h, cudaStreamCreateWithFlags(&wk.stream, cudaStreamNonBlocking));
  if (cublasCreate(&wk.cublas) != CUBLAS_STATUS_SUCCESS || cublasSetStream(wk.cublas, wk.stream) != CUBLAS_STATUS_SUCCESS ||
      cusolverDnCreate(&wk.cusolver) != CUSOLVER_STATUS_SUCCESS || cusolverDnSetStream(wk.cusolver, wk.stream) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnCreateParams(&wk.params) != CUSOLVER_STATUS_SUCCESS) {
    h->err = "eigensolver: creating the library handles of a Rayleigh-Ritz worker failed";
    return CX_ERR_LIB;
  }
  return CX_OK;
}

template <typename R>
static cx_status rayleigh_ritz_all(cx_handle h, int sel, int nmax, const std::vector<int>& off, double* EigVal) {
  const int nblk = h->nblk;
  if (h->rr_tier_n != nblk) {
    delete[] h->rr_tier;
    h->rr_tier = new int[nblk]();
    h->rr_tier_n = nblk;
  }
  const int nw = std::min(nblk, kRRWorkers);
  cx_status s;
  if (nw <= 1) {
    RRWork w{};
    if ((s = rr_workspace(h, nmax, nmax, w)) != CX_OK) return s;
    for (int b = 0; b < nblk; ++b)
      if ((s = rayleigh_ritz_block<R>(h, b, sel, w, EigVal + off[b])) != CX_OK) return s;
    return CX_OK;
  }
  while ((int)h->rr_workers.size() < nw) {
    h->rr_workers.emplace_back();
    if ((s = make_worker(h, h->rr_workers.back())) != CX_OK) return s;
  }
  cudaEvent_t ready;
  CX_TRY_CUDA(h, cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  CX_TRY_CUDA(h, cudaEventRecord(ready, h->stream));
  std::vector<cx_handle_s> shadow(nw, *h);
  std::vector<cx_status> st(nw, CX_OK);
  for (int i = 0; i < nw; ++i) {
    cx_rr_worker& wk = h->rr_workers[i];
    cx_handle_s& c = shadow[i];
    c.stream = wk.stream;
    c.cublas = wk.cublas;
    c.cusolver = wk.cusolver;
    c.cusolver_params = wk.params;
    c.d_ws = wk.d_ws; c.ws_bytes = wk.ws_bytes;
    c.h_ws = wk.h_ws; c.hws_bytes = wk.hws_bytes;
    c.d_rr = wk.d_rr; c.rr_bytes = wk.rr_bytes;
    c.launches = 0; c.eig_fallbacks = 0; c.eig_hermitian = 0; c.eig_restarts = 0;
    c.prof = false;
    CX_TRY_CUDA(h, cudaStreamWaitEvent(wk.stream, ready, 0));
  }
  std::vector<std::thread> threads;
  for (int i = 0; i < nw; ++i)
    threads.emplace_back([&, i]() {
      cx_handle c = &shadow[i];
      RRWork w{};
      st[i] = rr_workspace(c, nmax, nmax, w);
      for (int b = i; b < nblk && st[i] == CX_OK; b += nw) st[i] = rayleigh_ritz_block<R>(c, b, sel, w, EigVal + off[b]);
      if (cudaStreamSynchronize(c->stream) != cudaSuccess && st[i] == CX_OK) {
        c->err = "eigensolver: a Rayleigh-Ritz worker stream failed";
        st[i] = CX_ERR_CUDA;
      }
    });
  for (auto& t : threads) t.join();
  cudaEventDestroy(ready);
  s = CX_OK;
  for (int i = 0; i < nw; ++i) {
    cx_rr_worker& wk = h->rr_workers[i];
    const cx_handle_s& c = shadow[i];
    wk.d_ws = c.d_ws; wk.ws_bytes = c.ws_bytes;
    wk.h_ws = c.h_ws; wk.hws_bytes = c.hws_bytes;
    wk.d_rr = c.d_rr; wk.rr_bytes = c.rr_bytes;
    h->launches += c.launches;
    h->eig_fallbacks += c.eig_fallbacks;
    h->eig_hermitian += c.eig_hermitian;
    h->eig_restarts += c.eig_restarts;
    if (st[i] != CX_OK && s == CX_OK) {
      s = st[i];
      h->err = c.err;
    }
  }
  return s;
}

template <typename R>
static cx_status eigsolver_T(cx_handle h, const cx_eig_params& P, int count, double* ubgv, double* EigVal, double* a0, double* bup,
                             double* lc) {
  const int nblk = h->nblk, npl = P.npl;
  // subsequent relaxation steps filter with the current bounds from the first SCF cycle on
  // (src/eigSolver.m:21-23)
  const int elecgs = P.elecgs_Count < 1 ? 1 : P.elecgs_Count;
  const int rhoTrigger = elecgs > 1 ? 1 : P.rhoTrigger;
  h->restart_fail_streak = 0;
  CX_TRY_CUDA(h, cudaEventRecord(h->eig_ev[0], h->stream));
  std::vector<int> off(nblk + 1, 0);
  for (int b = 0; b < nblk; ++b) off[b + 1] = off[b] + h->blocks[b].Ns;
  auto min_ev = [&](int b) { return *std::min_element(EigVal + off[b], EigVal + off[b + 1]); };
  auto max_ev = [&](int b) { return *std::max_element(EigVal + off[b], EigVal + off[b + 1]); };
  // ---- bounds (src/eigSolver.m:47-84).  The upper bound is 1.01 x the largest Ritz value of a
  // Lanczos run; on the first relaxation step it starts from a random vector, later from the
  // previous upper-bound vector ubgv, whose update is returned in ubgv.
  const int K = 64;
  if (count == 1) {
    std::vector<double> lmin, lmax;
    cx_status s = lanczos_bounds<R>(h, K, lmin, lmax, elecgs > 1 ? ubgv : nullptr, ubgv);
    if (s != CX_OK) return s;
    for (int b = 0; b < nblk; ++b) {
      bup[b] = lmax[b] * 1.01;
      a0[b] = elecgs == 1 ? lmin[b] - 0.1 : min_ev(b);
    }
  } else if (count > rhoTrigger) {
    if (P.chefsibound_flag == 1) {
      std::vector<double> lmin, lmax;
      cx_status s = lanczos_bounds<R>(h, K, lmin, lmax, ubgv, ubgv);
      if (s != CX_OK) return s;
      for (int b = 0; b < nblk; ++b) bup[b] = lmax[b] * 1.01;
    }
    for (int b = 0; b < nblk; ++b) a0[b] = min_ev(b);
  }
  // ---- filter cutoff (src/eigSolver.m:88-94)
  std::vector<double> va(nblk), vb(nblk), va0(nblk);
  for (int b = 0; b < nblk; ++b) {
    lc[b] = (count == 1 && elecgs == 1) ? 0.5 * (bup[b] + a0[b]) : max_ev(b) + 0.10;
    va[b] = lc[b];
    vb[b] = bup[b];
    va0[b] = a0[b];
    if (!(vb[b] > va[b]) || !(va[b] > va0[b])) {
      h->err = "eigensolver: block " + std::to_string(b) + " has inconsistent bounds (need a0 < cutoff < bup)";
      return CX_ERR_ARG;
    }
  }
  // ---- Chebyshev filter of all blocks in one batched launch per degree
  size_t tot = 0;
  for (int b = 0; b < nblk; ++b) tot += (size_t)h->g.N * h->blocks[b].Ns;
  int sel = 0;
  cx_status s = filter_blocks<R>(h, (const BlockDev<R>*)h->d_blocks, nblk, h->d_state_tab, h->nstates, tot, h->psi_sel[0], npl, va,
                                 vb, va0, (cplx<R>*)h->d_cprime, &sel, h->d_maps ? &h->tma_main : nullptr);
  if (s != CX_OK) return s;
  // ---- H * X for all blocks (into the other buffer)
  {
    std::vector<StepScalars> one(nblk, StepScalars{1.0, 0.0, 0.0, 0.0});
    CX_TRY_CUDA(h, cudaMemcpyAsync(h->d_scal, one.data(), nblk * sizeof(StepScalars), cudaMemcpyHostToDevice, h->stream));
    s = fused_step<R>(h, (const BlockDev<R>*)h->d_blocks, h->d_scal, nblk, h->d_state_tab, h->nstates, sel, false,
                      (cplx<R>*)h->d_cprime, true, 2.0 * tot * sizeof(cplx<R>), h->d_maps ? &h->tma_main : nullptr);
    if (s != CX_OK) return s;
    if ((s = check_pipeline_status(h)) != CX_OK) return s;
  }
  // ---- Rayleigh-Ritz per block
  CX_TRY_CUDA(h, cudaEventRecord(h->eig_ev[1], h->stream));
  int nmax = 0;
  for (int b = 0; b < nblk; ++b) nmax = std::max(nmax, h->blocks[b].Ns);
  if ((s = rayleigh_ritz_all<R>(h, sel, nmax, off, EigVal)) != CX_OK) return s;
  h->psi_sel[0] = sel ^ 1;
  CX_TRY_CUDA(h, cudaEventRecord(h->eig_ev[2], h->stream));
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  // device time of the last call's parts: bounds + filter + H X, and the Rayleigh-Ritz steps
  float f_ms = 0, r_ms = 0;
  CX_TRY_CUDA(h, cudaEventElapsedTime(&f_ms, h->eig_ev[0], h->eig_ev[1]));
  CX_TRY_CUDA(h, cudaEventElapsedTime(&r_ms, h->eig_ev[1], h->eig_ev[2]));
  h->last_filter_ms = f_ms;
  h->last_rr_ms = r_ms;
  return CX_OK;
}

}  // namespace cx

using namespace cx;

// Device alias of page-locked host memory (registered or allocated page-locked), or null for
// pageable memory.  On Grace-Blackwell the GPU reads and writes such memory over NVLink-C2C, so the
// complex64 path converts straight between the caller's complex128 host array and the device
// buffer in one kernel, without a staging copy.
static void* mapped_alias(const void* host) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();                       // (pageable memory on older drivers reports an error)
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

cx_status cx_host_to_dev(cx_handle h, const double* host, void* dev, size_t n, int prec) {
  if (prec != CX_PREC_FP64) {
    if (const void* alias = mapped_alias(host)) {
      k_d2f<<<grid_for(n), 256, 0, h->stream>>>((const double2*)alias, (float2*)dev, n);
      h->launches++;
      CX_TRY_CUDA(h, cudaGetLastError());
      CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
      return CX_OK;
    }
  }
  if (prec == CX_PREC_FP64) {
    CX_TRY_CUDA(h, cudaMemcpyAsync(dev, host, n * 16, cudaMemcpyHostToDevice, h->stream));
    CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
    return CX_OK;
  }
  const size_t chunk = std::min<size_t>(n, (size_t)1 << 23);   // 128 MiB of complex128 per pass
  cx_status s = ensure(h, &h->d_stage, &h->stage_bytes, chunk * 16);
  if (s != CX_OK) return s;
  for (size_t o = 0; o < n; o += chunk) {
    const size_t m = std::min(chunk, n - o);
    CX_TRY_CUDA(h, cudaMemcpyAsync(h->d_stage, host + 2 * o, m * 16, cudaMemcpyHostToDevice, h->stream));
    k_d2f<<<grid_for(m), 256, 0, h->stream>>>((const double2*)h->d_stage, (float2*)dev + o, m);
    h->launches++;
  }
  CX_TRY_CUDA(h, cudaGetLastError());
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  return CX_OK;
}

cx_status cx_dev_to_host(cx_handle h, const void* dev, double* host, size_t n, int prec) {
  if (prec != CX_PREC_FP64) {
    if (void* alias = mapped_alias(host)) {
      k_f2d<<<grid_for(n), 256, 0, h->stream>>>((const float2*)dev, (double2*)alias, n);
      h->launches++;
      CX_TRY_CUDA(h, cudaGetLastError());
      CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
      return CX_OK;
    }
  }
  if (prec == CX_PREC_FP64) {
    CX_TRY_CUDA(h, cudaMemcpyAsync(host, dev, n * 16, cudaMemcpyDeviceToHost, h->stream));
    CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
    return CX_OK;
  }
  const size_t chunk = std::min<size_t>(n, (size_t)1 << 23);
  cx_status s = ensure(h, &h->d_stage, &h->stage_bytes, chunk * 16);
  if (s != CX_OK) return s;
  for (size_t o = 0; o < n; o += chunk) {
    const size_t m = std::min(chunk, n - o);
    k_f2d<<<grid_for(m), 256, 0, h->stream>>>((const float2*)dev + o, (double2*)h->d_stage, m);
    h->launches++;
    CX_TRY_CUDA(h, cudaMemcpyAsync(host + 2 * o, h->d_stage, m * 16, cudaMemcpyDeviceToHost, h->stream));
  }
  CX_TRY_CUDA(h, cudaGetLastError());
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  return CX_OK;
}

void cx_free_extra(cx_handle h) {
  cx::scf_state_free(h);
  for (auto& wk : h->rr_workers) {
    if (wk.stream) cudaStreamSynchronize(wk.stream);
    cudaFree(wk.d_ws);
    cudaFreeHost(wk.h_ws);
    cudaFree(wk.d_rr);
    if (wk.params) cusolverDnDestroyParams(wk.params);
    if (wk.cusolver) cusolverDnDestroy(wk.cusolver);
    if (wk.cublas) cublasDestroy(wk.cublas);
    if (wk.stream) cudaStreamDestroy(wk.stream);
  }
  h->rr_workers.clear();
  cudaFree(h->d_stage); h->d_stage = nullptr;
  cudaFree(h->d_rr); h->d_rr = nullptr;
  cudaFree(h->d_lz); h->d_lz = nullptr;
  cudaFree(h->d_misc); h->d_misc = nullptr;
  cudaFree(h->d_pois); h->d_pois = nullptr;
  cudaFree(h->d_scf); h->d_scf = nullptr;
  delete[] h->rr_tier;
  h->rr_tier = nullptr;
  h->rr_tier_n = 0;
}

// lambda_j = Re(sum W conj(a) b) / sum W |a|^2 for column j (one CTA per column)
__global__ void k_w_rq(const double2* __restrict__ A, const double2* __restrict__ HA, const double* __restrict__ W, int N,
                       double* __restrict__ lam) {
  const double2* a = A + (size_t)blockIdx.x * N;
  const double2* b = HA + (size_t)blockIdx.x * N;
  double num = 0, den = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    num += W[i] * (a[i].x * b[i].x + a[i].y * b[i].y);
    den += W[i] * (a[i].x * a[i].x + a[i].y * a[i].y);
  }
  __shared__ double r1[32], r2[32];
  for (int o = 16; o > 0; o >>= 1) { num += __shfl_xor_sync(0xffffffffu, num, o); den += __shfl_xor_sync(0xffffffffu, den, o); }
  if ((threadIdx.x & 31) == 0) { r1[threadIdx.x >> 5] = num; r2[threadIdx.x >> 5] = den; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double n1 = 0, d1 = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { n1 += r1[k]; d1 += r2[k]; }
    lam[blockIdx.x] = n1 / d1;
  }
}

namespace cx {
// Rayleigh quotients in FP64 of the device-resident psi of every block (see cx_refine_eigenvalues).
cx_status refine_eigenvalues(cx_handle h, double* EigVal) {
  const int N = h->g.N;
  int nmax = 0;
  for (int b = 0; b < h->nblk; ++b) nmax = std::max(nmax, h->blocks[b].Ns);
  const int nseg = std::max(1, h->nl.nseg);
  const size_t vec = (size_t)N * nmax * sizeof(double2);
  // two FP64 block buffers, projector coefficients, descriptors and the quotients
  double2 *A = nullptr, *HA = nullptr, *cp = nullptr;
  double* lam = nullptr;
  BlockDev<double>* d_blk = nullptr;
  int2* d_tab = nullptr;
  StepScalars* d_sc = nullptr;
  double2* d_ph = nullptr;
  cx_status s = CX_OK;
  auto fail = [&](const char* what) { h->err = std::string("cx_refine_eigenvalues: ") + what; s = CX_ERR_NOMEM; };
  if (cudaMalloc(&A, vec) != cudaSuccess || cudaMalloc(&HA, vec) != cudaSuccess ||
      cudaMalloc(&cp, (size_t)nmax * nseg * kAngMax * sizeof(double2)) != cudaSuccess || cudaMalloc(&lam, nmax * 8) != cudaSuccess ||
      cudaMalloc(&d_blk, sizeof(BlockDev<double>)) != cudaSuccess || cudaMalloc(&d_tab, nmax * sizeof(int2)) != cudaSuccess ||
      cudaMalloc(&d_sc, sizeof(StepScalars)) != cudaSuccess || cudaMalloc(&d_ph, nseg * sizeof(double2)) != cudaSuccess)
    fail("device buffers");
  int off = 0;
  for (int b = 0; s == CX_OK && b < h->nblk; ++b) {
    const int n = h->blocks[b].Ns;
    const void* psi = h->bufs[2 * b + h->psi_sel[0]];
    if (h->prec == CX_PREC_FP64) {
      if (cudaMemcpyAsync(A, psi, (size_t)N * n * 16, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess) { fail("copy"); break; }
    } else {
      k_f2d<<<grid_for((size_t)N * n), 256, 0, h->stream>>>((const float2*)psi, A, (size_t)N * n);
      h->launches++;
    }
    std::vector<BlockDev<double>> bd;
    make_block_devs<double>(h, std::vector<cplx<double>*>{A}, std::vector<cplx<double>*>{HA}, std::vector<int>{b}, bd);
    bd[0].Ns = n;
    std::vector<int2> tab(n);
    for (int i = 0; i < n; ++i) tab[i] = make_int2(0, i);
    const StepScalars one{1.0, 0.0, 0.0, 0.0};
    std::vector<double2> ph = segment_phases(h, h->blocks[b]);
    if (ph.empty()) ph.push_back(make_double2(1, 0));
    cudaMemcpyAsync(d_blk, bd.data(), sizeof(BlockDev<double>), cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(d_tab, tab.data(), n * sizeof(int2), cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(d_sc, &one, sizeof(one), cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(d_ph, ph.data(), ph.size() * sizeof(double2), cudaMemcpyHostToDevice, h->stream);
    const double2* saved = h->nl.seg_phase;
    const float2* saved32 = h->nl.seg_phase32;
    h->nl.seg_phase = d_ph;
    h->nl.seg_phase32 = nullptr;
    s = fused_step<double>(h, d_blk, d_sc, 1, d_tab, n, 0, false, cp, true, 0.0, nullptr);
    h->nl.seg_phase = saved;
    h->nl.seg_phase32 = saved32;
    if (s != CX_OK) break;
    k_w_rq<<<n, 256, 0, h->stream>>>(A, HA, h->d_W, N, lam);
    h->launches++;
    if (cudaMemcpyAsync(EigVal + off, lam, n * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      h->err = "cx_refine_eigenvalues: copy out";
      s = CX_ERR_CUDA;
      break;
    }
    off += n;
  }
  cudaStreamSynchronize(h->stream);
  cudaFree(A); cudaFree(HA); cudaFree(cp); cudaFree(lam); cudaFree(d_blk); cudaFree(d_tab); cudaFree(d_sc); cudaFree(d_ph);
  return s;
}

cx_status eigsolver_dispatch(cx_handle h, int count, int npl, int rhoTrigger, double* EigVal, double* a0, double* bup, double* lc) {
  const cx_eig_params P{npl, rhoTrigger, 1, 0};
  if (h->prec == CX_PREC_FP64) return eigsolver_T<double>(h, P, count, nullptr, EigVal, a0, bup, lc);
  return eigsolver_T<float>(h, P, count, nullptr, EigVal, a0, bup, lc);
}
}  // namespace cx

extern "C" {

cx_status cx_eigsolver_full(cx_handle h, const cx_eig_params* p, int32_t count, double* ubgv, double* EigVal, double* a0, double* bup,
                            double* lambda_cutoff) {
  if (!h) return CX_ERR_ARG;
  if (!p || !EigVal || !a0 || !bup || !lambda_cutoff) { h->err = "cx_eigsolver: null argument"; return CX_ERR_ARG; }
  if (h->nblk < 1) { h->err = "cx_eigsolver: call cx_set_blocks first"; return CX_ERR_STATE; }
  if (count < 1 || p->npl < 1) { h->err = "cx_eigsolver: need count >= 1 and npl >= 1"; return CX_ERR_ARG; }
  if (h->prec == CX_PREC_FP64) return eigsolver_T<double>(h, *p, count, ubgv, EigVal, a0, bup, lambda_cutoff);
  return eigsolver_T<float>(h, *p, count, ubgv, EigVal, a0, bup, lambda_cutoff);
}

cx_status cx_eigsolver(cx_handle h, int32_t count, int32_t npl, int32_t rhoTrigger, double* EigVal, double* a0, double* bup,
                       double* lambda_cutoff) {
  const cx_eig_params P{npl, rhoTrigger, 1, 0};
  return cx_eigsolver_full(h, &P, count, nullptr, EigVal, a0, bup, lambda_cutoff);
}

cx_status cx_refine_eigenvalues(cx_handle h, double* EigVal) {
  if (!h || !EigVal) return CX_ERR_ARG;
  if (h->nblk < 1) { h->err = "cx_refine_eigenvalues: call cx_set_blocks first"; return CX_ERR_STATE; }
  return cx::refine_eigenvalues(h, EigVal);
}

cx_status cx_eig_fallback_count(cx_handle h, int64_t* count) {
  if (!h || !count) return CX_ERR_ARG;
  *count = h->eig_fallbacks;
  return CX_OK;
}

cx_status cx_eig_hermitian_count(cx_handle h, int64_t* count) {
  if (!h || !count) return CX_ERR_ARG;
  *count = h->eig_hermitian;
  return CX_OK;
}

cx_status cx_eigsolver_full_host(cx_handle h, const cx_eig_params* p, int32_t count, double* ubgv, double* psi, double* EigVal,
                                 double* a0, double* bup, double* lambda_cutoff) {
  if (!h) return CX_ERR_ARG;
  if (!psi) { h->err = "cx_eigsolver_host: null psi"; return CX_ERR_ARG; }
  if (h->nblk < 1) { h->err = "cx_eigsolver_host: call cx_set_blocks first"; return CX_ERR_STATE; }
  size_t off = 0;
  for (int b = 0; b < h->nblk; ++b) {
    cx_status s = cx_set_psi(h, b, psi + 2 * off);
    if (s != CX_OK) return s;
    off += (size_t)h->g.N * h->blocks[b].Ns;
  }
  cx_status s = cx_eigsolver_full(h, p, count, ubgv, EigVal, a0, bup, lambda_cutoff);
  if (s != CX_OK) return s;
  off = 0;
  for (int b = 0; b < h->nblk; ++b) {
    s = cx_get_psi(h, b, psi + 2 * off);
    if (s != CX_OK) return s;
    off += (size_t)h->g.N * h->blocks[b].Ns;
  }
  return CX_OK;
}

cx_status cx_eigsolver_host(cx_handle h, int32_t count, int32_t npl, int32_t rhoTrigger, double* psi, double* EigVal, double* a0,
                            double* bup, double* lambda_cutoff) {
  const cx_eig_params P{npl, rhoTrigger, 1, 0};
  return cx_eigsolver_full_host(h, &P, count, nullptr, psi, EigVal, a0, bup, lambda_cutoff);
}

}  // extern "C"
