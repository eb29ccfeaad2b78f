// Rayleigh-Ritz products of the mixed-precision path on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), written for sm_103a without a library:
//
//   gram:    C = X^H (w .* Y)      X: N x n, Y: N x m complex64 (column-major), w: optional real
//                                  weights (N); C: n x m complex128: each CTA accumulates a short
//                                  range of the reduction in FP32 (tensor memory) and adds it to C
//                                  with FP64 atomics
//            (the Gram matrix X^H X, the projected Hamiltonian X^H (H X) and the W-Gram
//            X^H W X of src/eigSolver.m:99-104, in the Cholesky-QR form of this library);
//   rotate:  Z = X C               X: N x n complex64, C: n x m complex (FP64 in, split on the
//                                  device), Z: N x m complex64 (psi * Q of src/eigSolver.m:119).
//
// Precision: every FP32 operand a is split into a_hi = tf32(a) and a_lo = tf32(a - a_hi) (both
// rounded to nearest, so a_hi + a_lo represents a to 2^-22 relative); the products
// a_hi b_hi + a_hi b_lo + a_lo b_hi run as three kind::tf32 MMAs into one FP32 accumulator.  The
// dropped a_lo b_lo term and the representation leave a relative error of a few 2^-22 per
// product, unbiased: FP32-level products ("3xTF32").
//
// Complex arithmetic as real GEMMs (K-major operands, K = the reduction index):
//   gram:   with x^ = (re x_0, im x_0, re x_1, ...) and x~ = (-im x_0, re x_0, -im x_1, ...),
//           Re C_ij = x^_i . y^_j and Im C_ij = x~_i . y^_j over K = 2N: one MMA of M = 128 rows
//           (x^ of 64 columns of X, then x~ of the same 64) against N = 128 columns y^;
//   rotate: Re Z = Xr Cr - Xi Ci, Im Z = Xr Ci + Xi Cr over K = n: A = the real and imaginary
//           parts of 128 grid points of X (K-major after a register transpose), B = Cr^T, Ci^T
//           (64 columns of C); the minus sign is the MMA's negate-B bit.
//
// Data movement: 8 producer warps load the operands from global memory (coalesced), split them
// into hi / lo parts and store them in the no-swizzle K-major core-matrix layout (8 rows x 16 B
// per core matrix, 128 B apart along K, 1 KB apart along M/N); the rotation's C image is prepared
// once in that layout and copied per stage by cp.async.bulk.  One elected thread of a fifth warp
// issues the MMAs; stages are handed over by mbarriers (producers -> MMA: full, MMA commit ->
// producers: empty); the accumulator is read back with tcgen05.ld by the first 4 producer warps
// (warp w reads tensor-memory lanes 32 w .. 32 w + 31).
// Every wait is bounded: on a timeout the CTA records it in *status and skips to the end, where
// its tensor memory is released.
#include <algorithm>

#include "cx_common.h"

#include "cx_tc_helpers.cuh"

namespace cx {
namespace tc {

constexpr int kTileBytes = 128 * 128;   // 128 rows x 32 tf32 (K-major core matrices)

// ------------------------------------------------------------------------------------ gram
constexpr int kGramStages = 3;
constexpr int kGramXc = 64;      // X columns per tile (MMA M = 128: x^ and x~ rows)
constexpr int kGramN = 128;      // Y columns per tile (MMA N)
constexpr int kGramStageBytes = 4 * kTileBytes;   // A hi, A lo, B hi, B lo
constexpr size_t kGramSmem = 1024 + (size_t)kGramStages * kGramStageBytes;
// 8 producer warps (more global loads in flight per SM; the first 4 also read the accumulator back)
constexpr int kGramProducers = 8;
constexpr int kGramThreads = 32 * (kGramProducers + 1);
constexpr int kGramPieces = (kGramXc + kGramN) * 8 / (32 * kGramProducers);   // 16-byte pieces per producer thread and stage
static_assert((kGramXc + kGramN) * 8 % (32 * kGramProducers) == 0, "pieces per stage");

struct GramArgs {
  const float2* X;
  const float2* Y;
  const float* w;           // optional weights on Y (nullptr: none)
  double2* C;               // n x m, leading dimension ldc; accumulated in FP64 (zero it first)
  int N, n, m, ldc;
  int kchunk;               // complex grid points per split (multiple of 16)
  int* status;
};

__global__ void __launch_bounds__(kGramThreads, 1) gram_kernel(const __grid_constant__ GramArgs A) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)smem;                 // [stages]
  uint64_t* empty = full + kGramStages;             // [stages]
  uint64_t* done = empty + kGramStages;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  int* failed = (int*)(tmem_slot + 1);
  unsigned char* stages = smem + 1024;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = blockIdx.x * kGramXc, j0 = blockIdx.y * kGramN;
  const int kbeg = blockIdx.z * A.kchunk;
  const int kend = min(A.N, kbeg + A.kchunk);
  const int nk = kend > kbeg ? (kend - kbeg + 15) / 16 : 0;   // stages of 16 complex grid points

  if (threadIdx.x == 0) {
    for (int s = 0; s < kGramStages; ++s) {
      mbar_init(&full[s], 32 * kGramProducers);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, kGramN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < kGramProducers) {
    // ---- producers: 64 X columns and 128 Y columns x 16 complex grid points per stage, 16 B per
    // piece, kGramPieces pieces per thread.  The next stage's pieces are loaded into registers
    // before the current ones are split and stored, so a stage's global-load latency overlaps the
    // previous stage's work.
    const int t = threadIdx.x;
    auto load_stage = [&](int it, float4 (&v)[kGramPieces]) {
      const int kc0 = kbeg + 16 * it;
#pragma unroll
      for (int u = 0; u < kGramPieces; ++u) {
        const int pc = t + u * 32 * kGramProducers;
        const int col = pc >> 3, q = pc & 7;
        const int k = kc0 + 2 * q;
        const bool isx = col < kGramXc;
        const int c = isx ? i0 + col : j0 + (col - kGramXc);
        const float2* src = isx ? A.X : A.Y;
        float4 w4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < (isx ? A.n : A.m)) {
          const float2* colp = src + (size_t)c * A.N;
          if (k + 1 < kend && !(A.N & 1)) {
            w4 = *reinterpret_cast<const float4*>(colp + k);     // 16-byte aligned: N and k even
          } else if (k + 1 < kend) {
            const float2 e = colp[k], f = colp[k + 1];
            w4 = make_float4(e.x, e.y, f.x, f.y);
          } else if (k < kend) {
            const float2 e = colp[k];
            w4 = make_float4(e.x, e.y, 0.f, 0.f);
          }
          if (!isx && A.w) {
            const float w0 = k < kend ? A.w[k] : 0.f, w1 = k + 1 < kend ? A.w[k + 1] : 0.f;
            w4.x *= w0; w4.y *= w0; w4.z *= w1; w4.w *= w1;
          }
        }
        v[u] = w4;
      }
    };
    float4 cur[kGramPieces], nxt[kGramPieces];
    if (nk > 0) load_stage(0, cur);
    for (int it = 0; it < nk && !*(volatile int*)failed; ++it) {
      const int s = it % kGramStages;
      if (it + 1 < nk) load_stage(it + 1, nxt);
      if (it >= kGramStages && !mbar_wait(&empty[s], (uint32_t)(((it / kGramStages) - 1) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      unsigned char* Ahi = stages + (size_t)s * kGramStageBytes;
      unsigned char* Alo = Ahi + kTileBytes;
      unsigned char* Bhi = Alo + kTileBytes;
      unsigned char* Blo = Bhi + kTileBytes;
#pragma unroll
      for (int u = 0; u < kGramPieces; ++u) {
        const int pc = t + u * 32 * kGramProducers;
        const int col = pc >> 3, q = pc & 7;
        const float4 v = cur[u];
        float4 hi, lo;
        if (col < kGramXc) {
          split4(v, hi, lo);
          *reinterpret_cast<float4*>(Ahi + core_off(col, q)) = hi;
          *reinterpret_cast<float4*>(Alo + core_off(col, q)) = lo;
          split4(make_float4(-v.y, v.x, -v.w, v.z), hi, lo);     // x~ row
          *reinterpret_cast<float4*>(Ahi + core_off(col + kGramXc, q)) = hi;
          *reinterpret_cast<float4*>(Alo + core_off(col + kGramXc, q)) = lo;
        } else {
          split4(v, hi, lo);
          *reinterpret_cast<float4*>(Bhi + core_off(col - kGramXc, q)) = hi;
          *reinterpret_cast<float4*>(Blo + core_off(col - kGramXc, q)) = lo;
        }
      }
      fence_async_smem();
      mbar_arrive(&full[s]);
#pragma unroll
      for (int u = 0; u < kGramPieces; ++u) cur[u] = nxt[u];
    }
  } else if (lane == 0) {
    // ---- MMA issuer
    constexpr uint32_t idesc = idesc_tf32(128, kGramN, false);
    for (int it = 0; it < nk; ++it) {
      const int s = it % kGramStages;
      if (*(volatile int*)failed || !mbar_wait(&full[s], (uint32_t)((it / kGramStages) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      tc_fence_after();
      const uint32_t a_hi = su32(stages + (size_t)s * kGramStageBytes);
      const uint32_t a_lo = a_hi + kTileBytes, b_hi = a_lo + kTileBytes, b_lo = b_hi + kTileBytes;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {             // K = 8 per MMA: 2 core matrices of 4 values
        const uint32_t o = kk * 256;
        mma_tf32(tmem, smem_desc(a_hi + o, 128, 1024), smem_desc(b_hi + o, 128, 1024), idesc, (it | kk) != 0);
        mma_tf32(tmem, smem_desc(a_hi + o, 128, 1024), smem_desc(b_lo + o, 128, 1024), idesc, 1);
        mma_tf32(tmem, smem_desc(a_lo + o, 128, 1024), smem_desc(b_hi + o, 128, 1024), idesc, 1);
      }
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  // ---- epilogue: TMEM row m = 32 warp + lane -> Re (m < 64) or Im (m >= 64) of C[i0 + m % 64][j0 + .]
  if (warp < 4) {
    bool ok = nk > 0 && !*(volatile int*)failed;
    if (ok && !mbar_wait(done, 0)) {
      atomicExch(failed, 1);
      ok = false;
    }
    tc_fence_after();
    const int m = 32 * warp + lane;
    const int i = i0 + (m & 63), part = m >> 6;
    if (__any_sync(0xffffffffu, ok)) {
      for (int cb = 0; cb < kGramN / 16; ++cb) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(cb * 16), v);
        if (ok && i < A.n) {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int j = j0 + cb * 16 + e;
            if (j < A.m) atomicAdd(reinterpret_cast<double*>(A.C + (size_t)j * A.ldc + i) + part, (double)v[e]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && *failed) atomicExch(A.status, 1);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, kGramN);
  }
}

// ------------------------------------------------------------------------------------ rotate
constexpr int kRotStages = 2;
constexpr int kRotProducers = 8;                  // producer warps (the first 4 also read the accumulators back)
constexpr int kRotThreads = 32 * (kRotProducers + 1);
constexpr int kRotM = 128;       // grid points per tile
constexpr int kRotN = 64;        // columns of Z per tile (two accumulators: Re and Im)
constexpr int kRotATile = kRotM * 128;   // 128 rows x 32 tf32
constexpr int kRotBTile = kRotN * 128;   // 64 rows x 32 tf32
constexpr int kRotStageBytes = 4 * kRotATile + 4 * kRotBTile;   // A re/im hi/lo, B cr/ci hi/lo
constexpr size_t kRotSmem = 1024 + (size_t)kRotStages * kRotStageBytes;

struct RotArgs {
  const float2* X;          // N x n
  const float* Cimg;        // [jt][ks] blocks of 4 B tiles (Cr hi, Cr lo, Ci hi, Ci lo) in core-matrix layout
  float2* Z;                // N x m
  int N, n, m;
  int nks;                  // K stages (ceil(n / 32))
  int* status;
};

__global__ void __launch_bounds__(kRotThreads, 1) rotate_kernel(const __grid_constant__ RotArgs A) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)smem;
  uint64_t* empty = full + kRotStages;
  uint64_t* done = empty + kRotStages;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  int* failed = (int*)(tmem_slot + 1);
  unsigned char* stages = smem + 1024;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k0 = blockIdx.x * kRotM, jt = blockIdx.y, j0 = jt * kRotN;
  const int nk = A.nks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kRotStages; ++s) {
      mbar_init(&full[s], 32 * kRotProducers);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, 2 * kRotN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < kRotProducers) {
    // X: 128 grid points x 32 columns per stage; a warp task = 32 points (one per lane) x 4
    // columns, 4 tasks per warp.  The next stage's values are loaded into registers before the
    // current ones are split and stored (the load latency overlaps the previous stage's work).
    constexpr int kTasks = 32 / kRotProducers;
    auto load_stage = [&](int it, float2 (&v)[kTasks][4]) {
      const int ic0 = 32 * it;
#pragma unroll
      for (int u = 0; u < kTasks; ++u) {
        const int task = warp + u * kRotProducers;
        const int rb = task & 3, cq = task >> 2;          // row block of 32, column quad
        const int k = k0 + 32 * rb + lane;
        const int ib = ic0 + 4 * cq;
        const float2* xp = A.X + (size_t)ib * A.N + k;
#pragma unroll
        for (int e = 0; e < 4; ++e) v[u][e] = (k < A.N && ib + e < A.n) ? xp[(size_t)e * A.N] : make_float2(0.f, 0.f);
      }
    };
    float2 cur[kTasks][4], nxt[kTasks][4];
    if (nk > 0) load_stage(0, cur);
    for (int it = 0; it < nk && !*(volatile int*)failed; ++it) {
      const int s = it % kRotStages;
      if (it + 1 < nk) load_stage(it + 1, nxt);
      if (it >= kRotStages && !mbar_wait(&empty[s], (uint32_t)(((it / kRotStages) - 1) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      unsigned char* st = stages + (size_t)s * kRotStageBytes;
      // the stage's C tiles by one bulk copy, whose bytes the phase of full[s] waits for as well
      if (threadIdx.x == 0) {
        const float* src = A.Cimg + ((size_t)jt * A.nks + it) * (4 * kRotBTile / 4);
        mbar_expect_tx(&full[s], 4 * kRotBTile);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         su32(st + 4 * kRotATile)),
                     "l"(src), "r"((uint32_t)(4 * kRotBTile)), "r"(su32(&full[s]))
                     : "memory");
      }
#pragma unroll
      for (int u = 0; u < kTasks; ++u) {
        const int task = warp + u * kRotProducers;
        const int rb = task & 3, cq = task >> 2;
        const int r = 32 * rb + lane;
        const float4 re = make_float4(cur[u][0].x, cur[u][1].x, cur[u][2].x, cur[u][3].x);
        const float4 im = make_float4(cur[u][0].y, cur[u][1].y, cur[u][2].y, cur[u][3].y);
        float4 hi, lo;
        split4(re, hi, lo);
        *reinterpret_cast<float4*>(st + 0 * kRotATile + core_off(r, cq)) = hi;
        *reinterpret_cast<float4*>(st + 1 * kRotATile + core_off(r, cq)) = lo;
        split4(im, hi, lo);
        *reinterpret_cast<float4*>(st + 2 * kRotATile + core_off(r, cq)) = hi;
        *reinterpret_cast<float4*>(st + 3 * kRotATile + core_off(r, cq)) = lo;
      }
      fence_async_smem();
      mbar_arrive(&full[s]);
#pragma unroll
      for (int u = 0; u < kTasks; ++u)
#pragma unroll
        for (int e = 0; e < 4; ++e) cur[u][e] = nxt[u][e];
    }
  } else if (lane == 0) {
    constexpr uint32_t id_pos = idesc_tf32(kRotM, kRotN, false), id_neg = idesc_tf32(kRotM, kRotN, true);
    const uint32_t dre = tmem, dim = tmem + kRotN;
    for (int it = 0; it < nk; ++it) {
      const int s = it % kRotStages;
      if (*(volatile int*)failed || !mbar_wait(&full[s], (uint32_t)((it / kRotStages) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      tc_fence_after();
      const uint32_t base = su32(stages + (size_t)s * kRotStageBytes);
      const uint32_t xr_hi = base, xr_lo = base + kRotATile, xi_hi = base + 2 * kRotATile, xi_lo = base + 3 * kRotATile;
      const uint32_t cb = base + 4 * kRotATile;
      const uint32_t cr_hi = cb, cr_lo = cb + kRotBTile, ci_hi = cb + 2 * kRotBTile, ci_lo = cb + 3 * kRotBTile;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t o = kk * 256;
        auto d = [&](uint32_t a) { return smem_desc(a + o, 128, 1024); };
        const uint32_t first = (it | kk) != 0;
        // Re Z += Xr Cr - Xi Ci
        mma_tf32(dre, d(xr_hi), d(cr_hi), id_pos, first);
        mma_tf32(dre, d(xr_hi), d(cr_lo), id_pos, 1);
        mma_tf32(dre, d(xr_lo), d(cr_hi), id_pos, 1);
        mma_tf32(dre, d(xi_hi), d(ci_hi), id_neg, 1);
        mma_tf32(dre, d(xi_hi), d(ci_lo), id_neg, 1);
        mma_tf32(dre, d(xi_lo), d(ci_hi), id_neg, 1);
        // Im Z += Xr Ci + Xi Cr
        mma_tf32(dim, d(xr_hi), d(ci_hi), id_pos, first);
        mma_tf32(dim, d(xr_hi), d(ci_lo), id_pos, 1);
        mma_tf32(dim, d(xr_lo), d(ci_hi), id_pos, 1);
        mma_tf32(dim, d(xi_hi), d(cr_hi), id_pos, 1);
        mma_tf32(dim, d(xi_hi), d(cr_lo), id_pos, 1);
        mma_tf32(dim, d(xi_lo), d(cr_hi), id_pos, 1);
      }
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  if (warp < 4) {
    bool ok = nk > 0 && !*(volatile int*)failed;
    if (ok && !mbar_wait(done, 0)) {
      atomicExch(failed, 1);
      ok = false;
    }
    tc_fence_after();
    const int k = k0 + 32 * warp + lane;
    if (__any_sync(0xffffffffu, ok)) {
      for (int cb = 0; cb < kRotN / 16; ++cb) {
        float vr[16], vi[16];
        const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(cb * 16);
        tmem_ld16(ta, vr);
        tmem_ld16(ta + kRotN, vi);
        if (ok && k < A.N) {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int j = j0 + cb * 16 + e;
            if (j < A.m) A.Z[(size_t)j * A.N + k] = make_float2(vr[e], vi[e]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && *failed) atomicExch(A.status, 1);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * kRotN);
  }
}

// C (n x m complex128, column-major) -> per (column tile jt, K stage ks) the four B tiles Cr hi,
// Cr lo, Ci hi, Ci lo of 64 columns x 32 rows in the K-major core-matrix layout; zero outside C.
__global__ void k_rot_image(const double2* __restrict__ C, int n, int m, int nks, float* __restrict__ img) {
  const int njt = (m + kRotN - 1) / kRotN;
  const size_t per = (size_t)kRotN * 32;                   // values per tile
  const size_t tot = (size_t)njt * nks * per;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t blk = idx / per;
    const int e = (int)(idx % per);
    const int jr = e / 32, kr = e % 32;                    // row (column j of C) and K index within the tile
    const int jt = (int)(blk / nks), ks = (int)(blk % nks);
    const int j = jt * kRotN + jr, i = ks * 32 + kr;
    double2 c = make_double2(0.0, 0.0);
    if (i < n && j < m) c = C[(size_t)j * n + i];
    const float cr = (float)c.x, ci = (float)c.y;
    float hr, hi;
    {
      uint32_t r;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(cr));
      hr = __uint_as_float(r);
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(ci));
      hi = __uint_as_float(r);
    }
    float* base = img + blk * 4 * per;
    const uint32_t off = ((uint32_t)(jr >> 3) * 1024 + (uint32_t)(kr >> 2) * 128 + (uint32_t)(jr & 7) * 16) / 4 + (kr & 3);
    base[0 * per + off] = hr;
    base[1 * per + off] = tf32_hi(cr - hr);
    base[2 * per + off] = hi;
    base[3 * per + off] = tf32_hi(ci - hi);
  }
}

}  // namespace tc

// C (n x m, leading dimension ldc, complex128) = X^H (w .* Y); C is zeroed here.
cx_status tc_gram(cx_handle h, const float2* X, const float2* Y, const float* w, int N, int n, int m, double2* C, int ldc) {
  using namespace tc;
  CX_TRY_CUDA(h, cudaMemsetAsync(C, 0, (size_t)ldc * m * sizeof(double2), h->stream));
  if (N <= 0 || n <= 0 || m <= 0) return CX_OK;
  CX_TRY_CUDA(h, cudaFuncSetAttribute(gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGramSmem));
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = ((n + kGramXc - 1) / kGramXc) * ((m + kGramN - 1) / kGramN);
  // split the reduction over the grid points: short FP32 ranges (at most 1024 grid points, 2048
  // real terms, per CTA) and at least about two CTAs per SM
  int splits = std::max(1, (2 * nsm + tiles - 1) / tiles);
  int kchunk = (N + splits - 1) / splits;
  kchunk = std::min(kchunk, 1024);
  kchunk = std::max(16 * 8, (kchunk + 15) / 16 * 16);
  splits = (N + kchunk - 1) / kchunk;
  GramArgs a{X, Y, w, C, N, n, m, ldc, kchunk, h->d_status};
  dim3 grid((unsigned)((n + kGramXc - 1) / kGramXc), (unsigned)((m + kGramN - 1) / kGramN), (unsigned)splits);
  gram_kernel<<<grid, kGramThreads, kGramSmem, h->stream>>>(a);
  h->launches++;
  CX_TRY_CUDA(h, cudaGetLastError());
  return CX_OK;
}

// Z (N x m complex64) = X (N x n complex64) C (n x m complex128); img: scratch of
// tc_rot_image_floats(n, m) floats.
size_t tc_rot_image_floats(int n, int m) {
  using namespace tc;
  const size_t njt = (m + kRotN - 1) / kRotN, nks = (n + 31) / 32;
  return njt * nks * 4 * (size_t)kRotN * 32;
}
cx_status tc_rotate(cx_handle h, const float2* X, const double2* C, int N, int n, int m, float2* Z, float* img) {
  using namespace tc;
  if (N <= 0 || n <= 0 || m <= 0) return CX_OK;
  CX_TRY_CUDA(h, cudaFuncSetAttribute(rotate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRotSmem));
  const int nks = (n + 31) / 32;
  const size_t tot = tc_rot_image_floats(n, m) / 4;
  k_rot_image<<<(unsigned)std::min<size_t>((tot + 255) / 256, 152 * 16), 256, 0, h->stream>>>(C, n, m, nks, img);
  RotArgs a{X, img, Z, N, n, m, nks, h->d_status};
  dim3 grid((unsigned)((N + kRotM - 1) / kRotM), (unsigned)((m + kRotN - 1) / kRotN));
  rotate_kernel<<<grid, kRotThreads, kRotSmem, h->stream>>>(a);
  h->launches += 2;
  CX_TRY_CUDA(h, cudaGetLastError());
  return CX_OK;
}

}  // namespace cx
