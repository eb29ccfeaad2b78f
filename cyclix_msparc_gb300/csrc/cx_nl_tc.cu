// Kleinman-Bylander projector term of the complex64 path on the 5th-generation tensor cores
// (tcgen05.mma kind::tf32 with the 3xTF32 split of cx_tc_helpers.cuh, accumulators in tensor
// memory), written for sm_103a without a library:
//
//   contraction (src/h_nonlocal_vector_mult.m:24-37), one CTA per atom J and 64 states:
//       D[s, (img, q)] = sum over the ball nodes n of image img:  X[pos_n, s] (W Chi)[n, q]
//       C_J[s, q]      = sum_img p_img D[s, (img, q)]         (p = exp(i k.(R_J - R_img)) of the block)
//       C'[s, img, q]  = gamma_q conj(p_img) C_J[s, q]        (the apply's per-image coefficient)
//   apply (src/h_nonlocal_vector_mult.m:38-42), one CTA per 32-point row chunk and 64 states:
//       Y[chunk, s] += alpha_b Chi_c[32 x K] C'_c[K, s]        (K = 4 x the chunk's images)
//
// Both are real-by-complex products: the complex operand enters as 128 real rows (re and im of
// 64 states: MMA M = 128), the real Chi / W Chi as the B operand (N = the atom's image columns
// padded to 16, or the chunk's 32 points), K = ball nodes (32 per stage) or image columns (16 per
// stage).  The B operands do not change between calls: their hi / lo tf32 parts are laid out once
// on the host in the no-swizzle K-major core-matrix layout and copied per stage.  The complex
// operand is gathered, split and stored by 4 producer warps; one thread of a fifth warp issues
// the MMAs; the accumulator is read back by the producer warps.  The contraction needs no atomics
// (all nodes of an atom are reduced in one CTA), the apply none either (a chunk's points belong to
// one CTA).  Every wait is bounded: on a timeout the CTA records it in *status, skips its writes
// and releases its tensor memory.
#include <algorithm>
#include <cstring>

#include "cx_common.h"
#include "cx_tc_helpers.cuh"

namespace cx {
namespace tc {

constexpr int kNlProducerWarps = 4;
constexpr int kNlThreads = 32 * (kNlProducerWarps + 1);

// byte offset of row r, K-chunk c (4 values) in a K-major tile of kt K-values per row
__device__ __forceinline__ uint32_t core_off_k(int r, int c, int kt) {
  return (uint32_t)((r >> 3) * (kt * 32) + c * 128 + (r & 7) * 16);
}

// ------------------------------------------------------------------------------- contraction
constexpr int kCtK = 32;                         // ball nodes per stage
constexpr int kCtStages = 2;
constexpr int kCtNMax = 32;                      // image columns per atom (8 images)
constexpr int kCtATile = 128 * kCtK * 4;         // 16 KB
constexpr int kCtBTile = kCtNMax * kCtK * 4;     // 4 KB
constexpr int kCtStageBytes = 2 * kCtATile + 2 * kCtBTile;
constexpr size_t kCtSmem = 1024 + (size_t)kCtStages * kCtStageBytes;

struct NlContractArgs {
  const BlockDev<float>* blocks;
  const int2* state_tab;
  int nstates, N, in_sel, nseg;
  const int32_t* atom_node_ptr;   // n_atm + 1
  const int32_t* node_pos;        // 0-based grid index of each ball node
  const int32_t* atom_seg_ptr;    // n_atm + 1
  const int64_t* bimg_ptr;        // n_atm: float offset of the atom's B image
  const float* bimg;              // per atom: stages x (hi, lo) x NC x 32 tf32 values
  const double* gamma;            // n_atm x 4
  const float2* seg_phase32;      // nblk x nseg
  float2* cprime;                 // nstates x nseg x 4
  int* status;
};

__global__ void __launch_bounds__(kNlThreads, 2) nl_contract_tc_kernel(const __grid_constant__ NlContractArgs A) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)smem;
  uint64_t* empty = full + kCtStages;
  uint64_t* done = empty + kCtStages;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  int* failed = (int*)(tmem_slot + 1);
  unsigned char* stages = smem + 1024;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int J = blockIdx.x, g0 = blockIdx.y * 64;
  const int n0 = A.atom_node_ptr[J], n1 = A.atom_node_ptr[J + 1];
  const int s0 = A.atom_seg_ptr[J], nsJ = A.atom_seg_ptr[J + 1] - s0;
  if (nsJ <= 0) return;                          // no image reaches the cell: nothing to write
  const int NC = nsJ <= 4 ? 16 : 32;
  const int nk = (n1 - n0 + kCtK - 1) / kCtK;
  const float* bimg = A.bimg + A.bimg_ptr[J];

  if (threadIdx.x == 0) {
    for (int s = 0; s < kCtStages; ++s) {
      mbar_init(&full[s], 32 * kNlProducerWarps);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, 32);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < kNlProducerWarps) {
    // ---- producers.  A: piece (state j, node quad q) with j = t / 8 + 16 u, q = t % 8 (u < 4):
    // 4 gathered complex values -> 4 re values in row 2j and 4 im values in row 2j + 1.
    // B: the stage's image tiles (hi, lo: NC x 32 tf32 each) copied in 16-byte pieces.
    const int t = threadIdx.x, q = t & 7;
    const float2* colp[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int gs = g0 + (t >> 3) + 16 * u;
      colp[u] = nullptr;
      if (gs < A.nstates) {
        const int2 bs = A.state_tab[gs];
        colp[u] = A.blocks[bs.x].buf[A.in_sel] + (size_t)bs.y * A.N;
      }
    }
    const int nbq = NC * 16 / 128;               // 16-byte B pieces per thread (2 tiles x NC x 32 floats)
    auto load_stage = [&](int it, float2 (&v)[4][4], float4 (&b)[4]) {
      const int nb = n0 + it * kCtK + 4 * q;
      int pos[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) pos[i] = nb + i < n1 ? A.node_pos[nb + i] : -1;
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int i = 0; i < 4; ++i) v[u][i] = (colp[u] && pos[i] >= 0) ? colp[u][pos[i]] : make_float2(0.f, 0.f);
      const float4* src = reinterpret_cast<const float4*>(bimg + (size_t)it * 2 * NC * kCtK);
#pragma unroll
      for (int k = 0; k < 4; ++k) b[k] = k < nbq ? src[t + 128 * k] : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    float2 cur[4][4], nxt[4][4];
    float4 bc[4], bn[4];
    if (nk > 0) load_stage(0, cur, bc);
    for (int it = 0; it < nk && !*(volatile int*)failed; ++it) {
      const int s = it % kCtStages;
      if (it + 1 < nk) load_stage(it + 1, nxt, bn);
      if (it >= kCtStages && !mbar_wait(&empty[s], (uint32_t)(((it / kCtStages) - 1) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      unsigned char* Ahi = stages + (size_t)s * kCtStageBytes;
      unsigned char* Alo = Ahi + kCtATile;
      unsigned char* Bst = Alo + kCtATile;          // B hi tile, then B lo tile (NC rows each)
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = (t >> 3) + 16 * u;
        float4 hi, lo;
        split4(make_float4(cur[u][0].x, cur[u][1].x, cur[u][2].x, cur[u][3].x), hi, lo);
        *reinterpret_cast<float4*>(Ahi + core_off_k(2 * j, q, kCtK)) = hi;
        *reinterpret_cast<float4*>(Alo + core_off_k(2 * j, q, kCtK)) = lo;
        split4(make_float4(cur[u][0].y, cur[u][1].y, cur[u][2].y, cur[u][3].y), hi, lo);
        *reinterpret_cast<float4*>(Ahi + core_off_k(2 * j + 1, q, kCtK)) = hi;
        *reinterpret_cast<float4*>(Alo + core_off_k(2 * j + 1, q, kCtK)) = lo;
      }
      // the image holds the hi tile (NC x 32) then the lo tile: same byte layout in shared memory
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (k < nbq) {
          const int f = t + 128 * k;                // 16-byte piece of the two tiles
          const int tile = f / (NC * 8), off = f % (NC * 8);
          *reinterpret_cast<float4*>(Bst + (size_t)tile * kCtBTile + (size_t)off * 16) = bc[k];
        }
      }
      fence_async_smem();
      mbar_arrive(&full[s]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int i = 0; i < 4; ++i) cur[u][i] = nxt[u][i];
#pragma unroll
      for (int k = 0; k < 4; ++k) bc[k] = bn[k];
    }
  } else if (lane == 0) {
    // ---- MMA issuer: D[128 x NC] += A[128 x 32] B[NC x 32]^T per stage, 3xTF32
    const uint32_t idesc = idesc_tf32(128, NC, false);
    for (int it = 0; it < nk; ++it) {
      const int s = it % kCtStages;
      if (*(volatile int*)failed || !mbar_wait(&full[s], (uint32_t)((it / kCtStages) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      tc_fence_after();
      const uint32_t a_hi = su32(stages + (size_t)s * kCtStageBytes);
      const uint32_t a_lo = a_hi + kCtATile, b_hi = a_lo + kCtATile, b_lo = b_hi + kCtBTile;
#pragma unroll
      for (int kk = 0; kk < kCtK / 8; ++kk) {      // K = 8 per MMA: 2 core matrices of 4 values
        const uint32_t o = kk * 256;
        mma_tf32(tmem, smem_desc(a_hi + o, 128, kCtK * 32), smem_desc(b_hi + o, 128, kCtK * 32), idesc, (it | kk) != 0);
        mma_tf32(tmem, smem_desc(a_hi + o, 128, kCtK * 32), smem_desc(b_lo + o, 128, kCtK * 32), idesc, 1);
        mma_tf32(tmem, smem_desc(a_lo + o, 128, kCtK * 32), smem_desc(b_hi + o, 128, kCtK * 32), idesc, 1);
      }
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  // ---- epilogue: TMEM row m = 32 warp + lane -> state j = m / 2, re (m even) or im (m odd)
  if (warp < kNlProducerWarps) {
    bool ok = !*(volatile int*)failed;
    if (ok && nk > 0 && !mbar_wait(done, 0)) {
      atomicExch(failed, 1);
      ok = false;
    }
    tc_fence_after();
    float v[kCtNMax];
#pragma unroll
    for (int c = 0; c < kCtNMax; ++c) v[c] = 0.f;
    if (nk > 0 && __any_sync(0xffffffffu, ok)) {
      float w[16];
      tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), w);
#pragma unroll
      for (int c = 0; c < 16; ++c) v[c] = w[c];
      if (NC > 16) {
        tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 16u, w);
#pragma unroll
        for (int c = 0; c < 16; ++c) v[16 + c] = w[c];
      }
    }
    // both lanes of a pair get the complex row: (re, im) of every image column
    float o[kCtNMax];
#pragma unroll
    for (int c = 0; c < kCtNMax; ++c) o[c] = __shfl_xor_sync(0xffffffffu, v[c], 1);
    const int m = 32 * warp + lane, j = m >> 1, gs = g0 + j;
    const bool odd = lane & 1;
    if (ok && gs < A.nstates) {
      const int b = A.state_tab[gs].x;
      const float2* ph = A.seg_phase32 + (size_t)b * A.nseg + s0;
      // C_J[q] = sum_img p_img (re + i im)[img, q]
      float2 cj[4];
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) cj[qq] = make_float2(0.f, 0.f);
#pragma unroll
      for (int c = 0; c < kCtNMax; ++c) {
        const int img = c >> 2, qq = c & 3;
        if (img < nsJ) {
          const float re = odd ? o[c] : v[c], im = odd ? v[c] : o[c];
          const float2 p = ph[img];
          cj[qq].x += p.x * re - p.y * im;
          cj[qq].y += p.x * im + p.y * re;
        }
      }
      float gm[4];
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) gm[qq] = (float)A.gamma[(size_t)J * 4 + qq];
      // the pair splits the images: even lane the even ones, odd lane the odd ones
      float2* out = A.cprime + ((size_t)gs * A.nseg + s0) * 4;
      for (int img = odd ? 1 : 0; img < nsJ; img += 2) {
        const float2 p = ph[img];
        float4 w01, w23;
        float2 r[4];
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) {
          // gamma conj(p) C_J
          r[qq].x = gm[qq] * (p.x * cj[qq].x + p.y * cj[qq].y);
          r[qq].y = gm[qq] * (p.x * cj[qq].y - p.y * cj[qq].x);
        }
        w01 = make_float4(r[0].x, r[0].y, r[1].x, r[1].y);
        w23 = make_float4(r[2].x, r[2].y, r[3].x, r[3].y);
        reinterpret_cast<float4*>(out + (size_t)img * 4)[0] = w01;
        reinterpret_cast<float4*>(out + (size_t)img * 4)[1] = w23;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && *failed) atomicExch(A.status, 1);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 32);
  }
}

// ------------------------------------------------------------------------------------- apply
constexpr int kApK = 16;                         // image columns per stage (4 images)
constexpr int kApStages = 3;
constexpr int kApATile = 128 * kApK * 4;         // 8 KB
constexpr int kApBTile = 32 * kApK * 4;          // 2 KB
constexpr int kApStageBytes = 2 * kApATile + 2 * kApBTile;
constexpr size_t kApSmem = 1024 + (size_t)kApStages * kApStageBytes;

struct NlApplyArgs {
  const BlockDev<float>* blocks;
  const StepScalars* scal;
  const int2* state_tab;
  int nstates, N, Nx, out_sel, nseg;
  const int32_t* p0;              // first grid point of each chunk
  const int32_t* seg_ptr;         // nchunks + 1
  const int32_t* segs;            // image (segment) ids of each chunk
  const int64_t* bimg_ptr;        // per chunk: float offset of its B image
  const float* bimg;              // per chunk: stages x (hi, lo) x 32 x 16 tf32 values
  const float2* cprime;           // nstates x nseg x 4
  int* status;
};

__global__ void __launch_bounds__(kNlThreads, 3) nl_apply_tc_kernel(const __grid_constant__ NlApplyArgs A) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)smem;
  uint64_t* empty = full + kApStages;
  uint64_t* done = empty + kApStages;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  int* failed = (int*)(tmem_slot + 1);
  unsigned char* stages = smem + 1024;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x, g0 = blockIdx.y * 64;
  const int p0 = A.p0[c];
  const int sb = A.seg_ptr[c], nsc = A.seg_ptr[c + 1] - sb;
  const int nk = (nsc + 3) / 4;
  const float* bimg = A.bimg + A.bimg_ptr[c];

  if (threadIdx.x == 0) {
    for (int s = 0; s < kApStages; ++s) {
      mbar_init(&full[s], 32 * kNlProducerWarps);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, 32);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < kNlProducerWarps) {
    // ---- producers.  A: piece (state j, image slot l) with j = t / 4 + 32 u, l = t % 4 (u < 2):
    // the 4 coefficients of one image (32 B) -> 4 re values in row 2j, 4 im values in row 2j + 1.
    // B: the stage's hi and lo tiles (32 x 16 tf32 each), two 16-byte pieces per thread.
    const int t = threadIdx.x, l = t & 3;
    const float2* cs[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int gs = g0 + (t >> 2) + 32 * u;
      cs[u] = gs < A.nstates ? A.cprime + (size_t)gs * A.nseg * 4 : nullptr;
    }
    auto load_stage = [&](int it, float4 (&v)[2][2], float4 (&b)[2]) {
      const int li = it * 4 + l;
      const int sg = li < nsc ? A.segs[sb + li] : -1;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (cs[u] && sg >= 0) {
          const float4* p = reinterpret_cast<const float4*>(cs[u] + (size_t)sg * 4);
          v[u][0] = p[0];
          v[u][1] = p[1];
        } else {
          v[u][0] = v[u][1] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
      const float4* src = reinterpret_cast<const float4*>(bimg + (size_t)it * 2 * 32 * kApK);
      b[0] = src[t];
      b[1] = src[t + 128];
    };
    float4 cur[2][2], nxt[2][2], bc[2], bn[2];
    if (nk > 0) load_stage(0, cur, bc);
    for (int it = 0; it < nk && !*(volatile int*)failed; ++it) {
      const int s = it % kApStages;
      if (it + 1 < nk) load_stage(it + 1, nxt, bn);
      if (it >= kApStages && !mbar_wait(&empty[s], (uint32_t)(((it / kApStages) - 1) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      unsigned char* Ahi = stages + (size_t)s * kApStageBytes;
      unsigned char* Alo = Ahi + kApATile;
      unsigned char* Bst = Alo + kApATile;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int j = (t >> 2) + 32 * u;
        const float4 a = cur[u][0], bq = cur[u][1];   // (re0, im0, re1, im1), (re2, im2, re3, im3)
        float4 hi, lo;
        split4(make_float4(a.x, a.z, bq.x, bq.z), hi, lo);
        *reinterpret_cast<float4*>(Ahi + core_off_k(2 * j, l, kApK)) = hi;
        *reinterpret_cast<float4*>(Alo + core_off_k(2 * j, l, kApK)) = lo;
        split4(make_float4(a.y, a.w, bq.y, bq.w), hi, lo);
        *reinterpret_cast<float4*>(Ahi + core_off_k(2 * j + 1, l, kApK)) = hi;
        *reinterpret_cast<float4*>(Alo + core_off_k(2 * j + 1, l, kApK)) = lo;
      }
      // the image holds the hi tile then the lo tile (32 x 16 each): the shared-memory layout
      *reinterpret_cast<float4*>(Bst + (size_t)t * 16) = bc[0];
      *reinterpret_cast<float4*>(Bst + (size_t)(t + 128) * 16) = bc[1];
      fence_async_smem();
      mbar_arrive(&full[s]);
#pragma unroll
      for (int u = 0; u < 2; ++u) { cur[u][0] = nxt[u][0]; cur[u][1] = nxt[u][1]; }
      bc[0] = bn[0];
      bc[1] = bn[1];
    }
  } else if (lane == 0) {
    // ---- MMA issuer: D[128 x 32] += A[128 x 16] B[32 x 16]^T per stage, 3xTF32
    constexpr uint32_t idesc = idesc_tf32(128, 32, false);
    for (int it = 0; it < nk; ++it) {
      const int s = it % kApStages;
      if (*(volatile int*)failed || !mbar_wait(&full[s], (uint32_t)((it / kApStages) & 1))) {
        atomicExch(failed, 1);
        break;
      }
      tc_fence_after();
      const uint32_t a_hi = su32(stages + (size_t)s * kApStageBytes);
      const uint32_t a_lo = a_hi + kApATile, b_hi = a_lo + kApATile, b_lo = b_hi + kApBTile;
#pragma unroll
      for (int kk = 0; kk < kApK / 8; ++kk) {
        const uint32_t o = kk * 256;
        mma_tf32(tmem, smem_desc(a_hi + o, 128, kApK * 32), smem_desc(b_hi + o, 128, kApK * 32), idesc, (it | kk) != 0);
        mma_tf32(tmem, smem_desc(a_hi + o, 128, kApK * 32), smem_desc(b_lo + o, 128, kApK * 32), idesc, 1);
        mma_tf32(tmem, smem_desc(a_lo + o, 128, kApK * 32), smem_desc(b_hi + o, 128, kApK * 32), idesc, 1);
      }
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  // ---- epilogue: TMEM row m = 32 warp + lane -> state j = m / 2, re (m even) or im (m odd);
  // columns = the chunk's 32 points.  The pair exchanges halves: the even lane adds points 0-15,
  // the odd lane points 16-31 of state j.
  if (warp < kNlProducerWarps) {
    bool ok = nk > 0 && !*(volatile int*)failed;
    if (ok && !mbar_wait(done, 0)) {
      atomicExch(failed, 1);
      ok = false;
    }
    tc_fence_after();
    const int m = 32 * warp + lane, j = m >> 1, gs = g0 + j;
    const bool odd = lane & 1;
    if (__any_sync(0xffffffffu, ok)) {
      float v[32];
      {
        float w[16];
        tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), w);
#pragma unroll
        for (int e = 0; e < 16; ++e) v[e] = w[e];
        tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 16u, w);
#pragma unroll
        for (int e = 0; e < 16; ++e) v[16 + e] = w[e];
      }
      float2 y[16];
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const float send = odd ? v[e] : v[16 + e];
        const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
        y[e] = odd ? make_float2(recv, v[16 + e]) : make_float2(v[e], recv);
      }
      if (ok && gs < A.nstates) {
        const int2 bs = A.state_tab[gs];
        const float alpha = (float)A.scal[bs.x].alpha;
        const int row_end = (p0 / A.Nx + 1) * A.Nx;      // the chunk does not cross its theta-z row
        const int pb = p0 + (odd ? 16 : 0);
        const int npts = min(16, row_end - pb);
        float2* out = A.blocks[bs.x].buf[A.out_sel] + (size_t)bs.y * A.N + pb;
        if (npts == 16) {
#pragma unroll
          for (int e = 0; e < 16; e += 2) {
            float4 o = reinterpret_cast<float4*>(out)[e / 2];
            o.x = fmaf(alpha, y[e].x, o.x);
            o.y = fmaf(alpha, y[e].y, o.y);
            o.z = fmaf(alpha, y[e + 1].x, o.z);
            o.w = fmaf(alpha, y[e + 1].y, o.w);
            reinterpret_cast<float4*>(out)[e / 2] = o;
          }
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            if (e < npts) {
              float2 o = out[e];
              o.x = fmaf(alpha, y[e].x, o.x);
              o.y = fmaf(alpha, y[e].y, o.y);
              out[e] = o;
            }
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
    tmem_dealloc(tmem, 32);
  }
}

}  // namespace tc

// ---------------------------------------------------------------------------------- host side
// tf32 with round-to-nearest, ties away from zero (the device split's cvt.rna.tf32)
static float tf32_rna(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}
static void put_split(float* tile_hi, float* tile_lo, size_t idx, float x) {
  const float hi = tf32_rna(x);
  tile_hi[idx] = hi;
  tile_lo[idx] = tf32_rna(x - hi);
}

bool nl_tc_contract_images(const std::vector<int32_t>& atom_node_ptr, const std::vector<int32_t>& node_seg,
                           const std::vector<int32_t>& atom_seg_ptr, const std::vector<double>& node_wchi, std::vector<int64_t>& ptr,
                           std::vector<float>& img) {
  const int n_atm = (int)atom_node_ptr.size() - 1;
  ptr.assign(n_atm, 0);
  img.clear();
  for (int J = 0; J < n_atm; ++J) {
    const int n0 = atom_node_ptr[J], n1 = atom_node_ptr[J + 1];
    const int s0 = atom_seg_ptr[J], ns = atom_seg_ptr[J + 1] - s0;
    if (ns > tc::kCtNMax / kAngMax) return false;
    const int NC = ns <= 4 ? 16 : 32;
    const int nk = (n1 - n0 + tc::kCtK - 1) / tc::kCtK;
    ptr[J] = (int64_t)img.size();
    const size_t tile = (size_t)NC * tc::kCtK;
    img.resize(img.size() + (size_t)nk * 2 * tile, 0.f);
    float* base = img.data() + ptr[J];
    for (int it = 0; it < nk; ++it) {
      float* hi = base + (size_t)it * 2 * tile;
      float* lo = hi + tile;
      for (int i = 0; i < tc::kCtK; ++i) {
        const int n = n0 + it * tc::kCtK + i;
        if (n >= n1) break;
        const int ls = node_seg[n] - s0;
        for (int q = 0; q < kAngMax; ++q) {
          const int r = ls * kAngMax + q;
          const size_t idx = (size_t)(r >> 3) * (tc::kCtK * 8) + (size_t)(i >> 2) * 32 + (r & 7) * 4 + (i & 3);
          put_split(hi, lo, idx, (float)node_wchi[(size_t)n * kAngMax + q]);
        }
      }
    }
  }
  return true;
}

void nl_tc_apply_images(const std::vector<int32_t>& cseg_ptr, const std::vector<int64_t>& cchi_ptr, const std::vector<double>& cchi,
                        std::vector<int64_t>& ptr, std::vector<float>& img) {
  const int nch = (int)cseg_ptr.size() - 1;
  ptr.assign(nch, 0);
  img.clear();
  const size_t tile = (size_t)32 * tc::kApK;
  for (int c = 0; c < nch; ++c) {
    const int nsc = cseg_ptr[c + 1] - cseg_ptr[c];
    const int nk = (nsc + 3) / 4;
    ptr[c] = (int64_t)img.size();
    img.resize(img.size() + (size_t)nk * 2 * tile, 0.f);
    float* base = img.data() + ptr[c];
    for (int it = 0; it < nk; ++it) {
      float* hi = base + (size_t)it * 2 * tile;
      float* lo = hi + tile;
      for (int kk = 0; kk < tc::kApK; ++kk) {
        const int ls = it * 4 + kk / 4, q = kk % 4;
        if (ls >= nsc) continue;
        for (int r = 0; r < 32; ++r) {
          const size_t idx = (size_t)(r >> 3) * (tc::kApK * 8) + (size_t)(kk >> 2) * 32 + (r & 7) * 4 + (kk & 3);
          put_split(hi, lo, idx, (float)cchi[(size_t)cchi_ptr[c] + (size_t)(ls * kAngMax + q) * 32 + r]);
        }
      }
    }
  }
}

cudaError_t launch_nl_contract_tc(const GridDev& g, const BlockDev<float>* blocks, const int2* state_tab, int nstates, int in_sel,
                                  const NonlocalDev& nl, const NlTcImages& im, float2* cprime, int* status, cudaStream_t st) {
  if (nl.n_atm == 0 || nstates == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(tc::nl_contract_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kCtSmem);
  if (e != cudaSuccess) return e;
  tc::NlContractArgs a{};
  a.blocks = blocks;
  a.state_tab = state_tab;
  a.nstates = nstates;
  a.N = g.N;
  a.in_sel = in_sel;
  a.nseg = nl.nseg;
  a.atom_node_ptr = nl.atom_node_ptr;
  a.node_pos = nl.node_pos;
  a.atom_seg_ptr = nl.atom_seg_ptr;
  a.bimg_ptr = im.ct_ptr;
  a.bimg = im.ct_img;
  a.gamma = nl.gamma;
  a.seg_phase32 = nl.seg_phase32;
  a.cprime = cprime;
  a.status = status;
  dim3 grid((unsigned)nl.n_atm, (unsigned)((nstates + 63) / 64));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  tc::nl_contract_tc_kernel<<<grid, tc::kNlThreads, tc::kCtSmem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_nl_apply_tc(const GridDev& g, const BlockDev<float>* blocks, const StepScalars* scal, const int2* state_tab,
                               int nstates, int out_sel, const ChunkTables& ct, const NlTcImages& im, const float2* cprime, int nseg,
                               int* status, cudaStream_t st) {
  if (ct.nchunks == 0 || nseg == 0 || nstates == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(tc::nl_apply_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kApSmem);
  if (e != cudaSuccess) return e;
  tc::NlApplyArgs a{};
  a.blocks = blocks;
  a.scal = scal;
  a.state_tab = state_tab;
  a.nstates = nstates;
  a.N = g.N;
  a.Nx = g.Nx;
  a.out_sel = out_sel;
  a.nseg = nseg;
  a.p0 = ct.p0;
  a.seg_ptr = ct.seg_ptr;
  a.segs = ct.segs;
  a.bimg_ptr = im.ap_ptr;
  a.bimg = im.ap_img;
  a.cprime = cprime;
  a.status = status;
  dim3 grid((unsigned)ct.nchunks, (unsigned)((nstates + 63) / 64));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  tc::nl_apply_tc_kernel<<<grid, tc::kNlThreads, tc::kApSmem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace cx
