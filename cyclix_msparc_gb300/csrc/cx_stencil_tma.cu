// TMA-pipelined fused H*psi / Chebyshev step for complex64 blocks (the production path of the
// mixed-precision filter).  Same arithmetic as cheb_step_kernel in cx_stencil.cu
// (Cychel/lapVec_cychel.m:19-52, src/h_nonlocal_vector_mult.m:21, src/chebyshev_filter.m:24-42),
// different data movement:
//
//  * a CTA owns TR = 32 radial points x TY theta rows of one state (all Ny rows when they fit,
//    else Ny / TY row tiles) and marches along z over a chunk of output planes;
//  * every z-plane of the tile is copied HBM -> shared memory once by cp.async.bulk.tensor.4d into
//    a ring of 1 + P stages guarded by mbarriers: the TY rows (+ FDn radial halo each side,
//    zero-filled by TMA outside [0, Nr): the Dirichlet walls) between theta halo rows, and the
//    plane's Veff tile (float copy).  With one theta tile the halo rows are copies of the tile's
//    own rows times the Bloch phase, made in shared memory one plane ahead; with several tiles
//    two more copies bring 8-row halos and the wrapping ones are multiplied by the phase in
//    place.  Every thread reads straight theta windows (no per-element wrap logic, all warps do
//    the same work);
//  * each plane is used once, when it arrives: its in-plane part (radial + theta + Veff) goes to
//    the accumulator of the same output plane and its z-stencil contributions are forwarded to
//    the accumulators of the 2 FDn planes around it.  Each thread keeps 2 FDn + 1 pending output
//    accumulators in registers; slot k holds output plane z - FDn + k, and the shift to the next
//    plane is folded into the multiply-adds (slot k <- slot k+1 + c x), so register indices stay
//    compile-time with no branch;
//  * helical cells: the cross term (X DG2^T) DG3^T equals D_z (D_theta X) (the two 1-D operators
//    act on different indices and commute); D_theta of the arriving plane is formed from the
//    same theta window and forwarded like the z-stencil terms;
//  * P (planes in flight) is as deep as shared memory allows;
//  * complex values are (re, im) register pairs and all arithmetic on them is packed
//    f32x2 (fma.rn.f32x2 / add.rn.f32x2): one instruction per complex-by-real term;
//  * the previous Chebyshev iterate of each output plane arrives by TMA in a second ring;
//  * the Kleinman-Bylander term is not part of this kernel: nl_apply_kernel (cx_stencil.cu) adds it
//    afterwards on the 32-point row chunks that a projector ball touches;
//  * mbarrier waits are bounded; on a timeout the CTA records it in *status, drains its own
//    outstanding copies (again bounded) and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "cx_common.h"

namespace cx {

constexpr int TM_F = 6;        // FD half-width this kernel is written for (FD order 12)
constexpr int TM_Q = 2 * TM_F + 1;
constexpr int TM_TR = 32;      // radial points per tile (one per lane)
constexpr int TM_BW = TM_TR + 2 * TM_F;   // staged row width (complex64), 352 B
constexpr int TM_HALO = 8;     // theta halo rows staged above / below the tile (FDn used)
constexpr int TM_PMAX = 8;     // X planes prefetched ahead of the consumer, at most
constexpr int TM_MAXW = 12;    // warps per CTA at most with 2 or 3 rows per thread (register budget of 12 warps)
constexpr int TM_MAXW1 = 16;   // warps per CTA at most with one row per thread
constexpr size_t TM_SMEM_MAX = 200 * 1024;

struct TmaArgs {
  GridDev g;
  const BlockDev<float>* blocks;
  const StepScalars* scal;
  const int2* state_tab;
  const CUtensorMap* xmaps;     // [block][buffer], box = TM_BW x TY
  const CUtensorMap* hmaps;     // [block][buffer], box = TM_BW x TM_HALO
  const CUtensorMap* omaps;     // [block][buffer], box = 32 x TY
  const CUtensorMap* vmaps;     // [spin] float Veff, box = 32 x TY
  int* status;
  int tiles_r, tiles_t, TY, in_sel, use_xprev;
  int full_items, zsplit;       // work items [0, full_items) cover all of z; the rest split z in zsplit chunks
  int stage_bytes, nst, ostage_bytes, nos;    // X stages (rows + Veff tile), xprev stages
  float cr2[TM_F + 1], cr1[TM_F + 1], ct2[TM_F + 1], ct1[TM_F + 1], cz2[TM_F + 1], cz1[TM_F + 1];
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: true when the phase completed, false after about a second (2^31 SM cycles)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t_end = clock64() + (1LL << 31);
  while (clock64() < t_end)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(su32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(su32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(su32(dst)),
               "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(su32(bar))
               : "memory");
}

// ---- packed f32x2 arithmetic on (re, im) pairs (sm_100-family FFMA2 / FADD2 / FMUL2)
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }   // a * b + c
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 dup2(float c) { return make_float2(c, c); }
__device__ __forceinline__ float2 cmulf(float2 v, float2 p) {
  return make_float2(v.x * p.x - v.y * p.y, v.x * p.y + v.y * p.x);
}

// Forward the contributions of the arriving plane z for one row.  Register slot k holds the
// pending output plane z - F + k, so moving on by one plane is a shift of the slots, folded into
// the multiply-adds (slot k <- slot k+1 + cz2[|k - F|] x, in place in ascending k; compile-time
// register indices, no branch):
//   slot 2F starts with cz2[F] x,  slot F (output z) takes the in-plane part, which holds the
//   centre coefficient cz2[0] with the other centre terms,
//   helical: output z - q gets + cz1[q] v and output z + q gets - cz1[q] v, with v = D_theta x;
// slot 0 (output z - F) is then complete and returned.
template <bool HEL>
__device__ __forceinline__ float2 forward_row(float2 (&acc)[TM_Q], float2 x, float2 inp, float2 vth, bool is_out,
                                              const float* __restrict__ cz2, const float* __restrict__ cz1) {
  constexpr int F = TM_F, Q = TM_Q;
#pragma unroll
  for (int k = 0; k < Q - 1; ++k) {
    const int d = k - F;                   // this slot's output plane is z + d
    if (d == 0) {
      acc[k] = acc[k + 1];                 // the centre cz2[0] x is part of the in-plane term
    } else {
      acc[k] = f2fma(dup2(cz2[d < 0 ? -d : d]), x, acc[k + 1]);
      if (HEL) acc[k] = f2fma(dup2(d < 0 ? cz1[-d] : -cz1[d]), vth, acc[k]);
    }
  }
  acc[Q - 1] = f2mul(dup2(cz2[F]), x);
  if (HEL) acc[Q - 1] = f2fma(dup2(-cz1[F]), vth, acc[Q - 1]);
  if (is_out) acc[F] = f2add(acc[F], inp);
  return acc[0];
}

// RPT: theta rows per thread, HEL: helical cross term
template <int RPT, bool HEL>
__global__ void __launch_bounds__((RPT == 1 ? TM_MAXW1 : TM_MAXW) * 32, 1) cheb_tma_kernel(const __grid_constant__ TmaArgs A) {
  constexpr int F = TM_F, Q = TM_Q, BW = TM_BW, H = TM_HALO;
  extern __shared__ __align__(128) unsigned char smem[];
  const int Nx = A.g.Nx, Ny = A.g.Ny, Nz = A.g.Nz;
  const int NST = A.nst, NOS = A.nos, TY = A.TY;
  uint64_t* full = (uint64_t*)smem;                                       // NST barriers (X ring)
  uint64_t* ofull = full + 16;                                            // NOS barriers (xprev ring)
  unsigned char* ring = smem + 256;
  unsigned char* oring = ring + (size_t)NST * A.stage_bytes;
  const int rows_bytes = BW * (TY + 2 * H) * 8;                            // the Veff tile follows the rows

  const int lane = threadIdx.x & 31;
  const int wy = threadIdx.x >> 5;
  // work item of this CTA: (state, r tile, theta tile, z range).  The last, partial wave of
  // whole-z items is split along z so that it spreads over all SMs.
  const int per_state = A.tiles_r * A.tiles_t;
  int item, z0, z1;
  if ((int)blockIdx.x < A.full_items) {
    item = blockIdx.x;
    z0 = 0;
    z1 = Nz;
  } else {
    const int j = blockIdx.x - A.full_items;
    const int c = j % A.zsplit;
    item = A.full_items + j / A.zsplit;
    z0 = (int)((long)c * Nz / A.zsplit);
    z1 = (int)((long)(c + 1) * Nz / A.zsplit);
  }
  const int gs = item / per_state;
  const int ir = (item % per_state) % A.tiles_r;
  const int itl = (item % per_state) / A.tiles_r;
  const int2 bs = A.state_tab[gs];
  const BlockDev<float>& B = A.blocks[bs.x];
  const size_t plane = (size_t)Nx * Ny;
  const size_t sN = (size_t)bs.y * plane * Nz;
  float2* __restrict__ out = B.buf[A.in_sel ^ 1] + sN;
  const float2 ph_tl = make_float2((float)B.ph_tl.x, (float)B.ph_tl.y), ph_tr = make_float2((float)B.ph_tr.x, (float)B.ph_tr.y);
  const float2 ph_zl = make_float2((float)B.ph_zl.x, (float)B.ph_zl.y), ph_zr = make_float2((float)B.ph_zr.x, (float)B.ph_zr.y);
  const StepScalars sc = A.scal[bs.x];
  const float alpha = (float)sc.alpha, cshift = (float)sc.c, beta = (float)sc.beta;
  const CUtensorMap* xmap = A.xmaps + 2 * bs.x + A.in_sel;
  const CUtensorMap* hmap = A.hmaps + 2 * bs.x + A.in_sel;
  const CUtensorMap* omap = A.omaps + 2 * bs.x + (A.in_sel ^ 1);
  const CUtensorMap* vmap = A.vmaps + B.veff_spin;
  const bool bcz = A.g.BCz != 0;

  const int r0 = ir * TM_TR;
  const int t0 = itl * TY;
  const int zstart = z0 - F;
  const int nplanes = z1 + F - zstart;
  const int nout = z1 - z0;
  // theta halo rows: above the tile rows t0-H..t0-1, below t0+TY..t0+TY+H-1 (mod Ny)
  const bool one_tile = A.tiles_t == 1;
  const int t_top = t0 == 0 ? Ny - H : t0 - H;
  const int t_bot = t0 + TY == Ny ? 0 : t0 + TY;
  const bool ph_top_on = ph_tl.x != 1.f || ph_tl.y != 0.f, ph_bot_on = ph_tr.x != 1.f || ph_tr.y != 0.f;
  const bool fix_top = !one_tile && t0 == 0 && ph_top_on;
  const bool fix_bot = !one_tile && t0 + TY == Ny && ph_bot_on;
  const bool fix_z = ph_zl.x != 1.f || ph_zl.y != 0.f;

  const int r = r0 + lane;
  const bool rok = r < Nx;
  const double rr = A.g.xin + (double)r * A.g.dx;
  const float inv_r = (float)(1.0 / rr);
  const float th_scale = HEL ? (float)(A.g.twist * A.g.twist + 1.0 / (rr * rr)) : (float)(1.0 / (rr * rr));
  float2 cp[F + 1], cm[F + 1];
#pragma unroll
  for (int q = 1; q <= F; ++q) {
    cp[q] = dup2(A.cr2[q] + inv_r * A.cr1[q]);
    cm[q] = dup2(A.cr2[q] - inv_r * A.cr1[q]);
  }
  // centre coefficient of the Laplacian minus the 2 (Veff - c) term (added per point)
  const float c0 = A.cr2[0] + th_scale * A.ct2[0] + A.cz2[0] + 2.f * cshift;
  const float2 ths = dup2(th_scale);
  const float2 mhalf_alpha = dup2(-0.5f * alpha);
  const int col = lane + F;
  const uint32_t xbytes = (uint32_t)(BW * (one_tile ? TY : TY + 2 * H) * 8 + 32 * TY * 4);
  const uint32_t obytes = (uint32_t)(32 * TY * 8);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) mbar_init(&full[s], 1);
    for (int s = 0; s < NOS; ++s) mbar_init(&ofull[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue_x = [&](int it) {             // X plane zstart + it (rows, halos, Veff) into stage it % NST
    const int s = it % NST;
    int zc = zstart + it;
    if (!bcz) { if (zc < 0) zc += Nz; else if (zc >= Nz) zc -= Nz; }
    unsigned char* dst = ring + (size_t)s * A.stage_bytes;
    mbar_expect_tx(&full[s], xbytes);
    if (!one_tile) tma_load_4d(dst, hmap, &full[s], r0 - F, t_top, zc, bs.y);
    tma_load_4d(dst + (size_t)H * BW * 8, xmap, &full[s], r0 - F, t0, zc, bs.y);
    if (!one_tile) tma_load_4d(dst + (size_t)(H + TY) * BW * 8, hmap, &full[s], r0 - F, t_bot, zc, bs.y);
    if (bcz && (zc < 0 || zc >= Nz)) zc = 0;   // Veff of a Dirichlet ghost plane is never used
    tma_load_3d(dst + rows_bytes, vmap, &full[s], r0, t0, zc);
  };
  auto issue_o = [&](int io) {             // previous iterate of output plane z0 + io into stage io % NOS
    const int s = io % NOS;
    unsigned char* dst = oring + (size_t)s * A.ostage_bytes;
    mbar_expect_tx(&ofull[s], obytes);
    tma_load_4d(dst, omap, &ofull[s], r0, t0, z0 + io, bs.y);
  };
  // theta halo rows of the plane in stage s (one tile: phased copies of the tile's own rows;
  // several tiles: the Bloch phase on the staged rows that wrap)
  auto prep_halo = [&](int s) {
    float2* P = (float2*)(ring + (size_t)s * A.stage_bytes);
    constexpr int BW4 = BW / 2;            // 16-byte pieces (two complex values) per staged row
    if (one_tile) {
      // halo rows -F..-1 (k < F) and Ny..Ny+F-1 (k >= F), two complex values per thread and step
      for (int i = threadIdx.x; i < 2 * F * BW4; i += blockDim.x) {
        const int k = i / BW4, c = 2 * (i - k * BW4);
        const bool top = k < F;
        const int dst_row = top ? H - F + k : H + Ny + (k - F);
        const int src_row = top ? H + Ny - F + k : H + (k - F);
        const bool ph = top ? ph_top_on : ph_bot_on;
        const float2 p = top ? ph_tl : ph_tr;
        const float4 v = *reinterpret_cast<const float4*>(P + (size_t)src_row * BW + c);
        float4 o = v;
        if (ph) {
          const float2 a = cmulf(make_float2(v.x, v.y), p), b = cmulf(make_float2(v.z, v.w), p);
          o = make_float4(a.x, a.y, b.x, b.y);
        }
        *reinterpret_cast<float4*>(P + (size_t)dst_row * BW + c) = o;
      }
    } else if (fix_top || fix_bot) {
      for (int i = threadIdx.x; i < 2 * H * BW4; i += blockDim.x) {
        const int k = i / BW4, c = 2 * (i - k * BW4);
        const bool top = k < H;
        if (top ? fix_top : fix_bot) {
          float4* q = reinterpret_cast<float4*>(P + (size_t)(top ? k : H + TY + (k - H)) * BW + c);
          const float2 p = top ? ph_tl : ph_tr;
          const float4 v = *q;
          const float2 a = cmulf(make_float2(v.x, v.y), p), b = cmulf(make_float2(v.z, v.w), p);
          *q = make_float4(a.x, a.y, b.x, b.y);
        }
      }
    }
  };

  int issued = 0, oissued = 0;
  if (threadIdx.x == 0) {
    const int n0 = min(NST, nplanes);
    for (int k = 0; k < n0; ++k) issue_x(k);
    issued = n0;
    if (A.use_xprev) {
      const int m0 = min(NOS, nout);
      for (int k = 0; k < m0; ++k) issue_o(k);
      oissued = m0;
    }
  }

  float2 acc[RPT][Q];
#pragma unroll
  for (int j = 0; j < RPT; ++j)
#pragma unroll
    for (int k = 0; k < Q; ++k) acc[j][k] = make_float2(0.f, 0.f);

  bool failed = false;
  int waited = 0, ocur = 0;                // planes / xprev tiles whose arrival was awaited
  if (!mbar_wait_bounded(&full[0], 0u)) failed = true;
  waited = 1;
  prep_halo(0);
  if (__syncthreads_or(failed)) failed = true;
  int s = 0, par = 0;                      // X-ring stage and parity of plane `it`
  int os = 0, opar = 0;                    // xprev-ring stage and parity
  for (int it = 0; it < nplanes && !failed; ++it) {
    // the next plane: wait for it and build its halo rows first, so that their shared-memory
    // round trips overlap this plane's arithmetic (nobody reads them before the barrier below)
    int s1 = s + 1, par1 = par;
    if (s1 == NST) { s1 = 0; par1 ^= 1; }
    if (it + 1 < nplanes) {
      if (!mbar_wait_bounded(&full[s1], (uint32_t)par1)) failed = true;
      waited = it + 2;
      prep_halo(s1);
    }
    const int zi = zstart + it;
    const float2* P = (const float2*)(ring + (size_t)s * A.stage_bytes);
    const float* Vt = (const float*)(ring + (size_t)s * A.stage_bytes + rows_bytes);
    const bool is_out = zi >= z0 && zi < z1;
    const bool zw = !bcz && fix_z && (zi < 0 || zi >= Nz);
    const float2 pz = zi < 0 ? ph_zl : ph_zr;
    // theta window of this thread's rows: rows wy*RPT-F .. wy*RPT+RPT-1+F of the arriving plane
    float2 w[RPT + 2 * F];
#pragma unroll
    for (int k = 0; k < RPT + 2 * F; ++k) w[k] = P[(size_t)(H + wy * RPT - F + k) * BW + col];
    float2 xv[RPT], inp[RPT], vth[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
      const int t = wy * RPT + j;
      xv[j] = zw ? cmulf(w[j + F], pz) : w[j + F];
      inp[j] = make_float2(0.f, 0.f);
      vth[j] = make_float2(0.f, 0.f);
      if (is_out) {
        // radial: (DL11 + DG1) with the 1/r first-derivative folded into the coefficients
        // (two independent chains: + and - neighbours)
        const float2* row = P + (size_t)(H + (t < TY ? t : 0)) * BW + col;
        float2 rp = f2mul(cp[1], row[1]);
        float2 rm = f2mul(cm[1], row[-1]);
#pragma unroll
        for (int q = 2; q <= F; ++q) {
          rp = f2fma(cp[q], row[q], rp);
          rm = f2fma(cm[q], row[-q], rm);
        }
        // theta: two chains (odd / even q)
        float2 ta = f2mul(dup2(A.ct2[1]), f2add(w[j + F + 1], w[j + F - 1]));
        float2 tb = f2mul(dup2(A.ct2[2]), f2add(w[j + F + 2], w[j + F - 2]));
#pragma unroll
        for (int q = 3; q <= F; q += 2) {
          ta = f2fma(dup2(A.ct2[q]), f2add(w[j + F + q], w[j + F - q]), ta);
          tb = f2fma(dup2(A.ct2[q + 1]), f2add(w[j + F + q + 1], w[j + F - q - 1]), tb);
        }
        const float v = Vt[(t < TY ? t : 0) * 32 + lane];
        inp[j] = f2fma(ths, f2add(ta, tb), f2fma(dup2(c0 - 2.f * v), xv[j], f2add(rp, rm)));
      }
      if (HEL) {
        // D_theta of the arriving plane: sum_q ct1[q] (w[t+q] - w[t-q])
        float2 da = f2mul(dup2(A.ct1[1]), w[j + F + 1]);
        float2 db = f2mul(dup2(-A.ct1[1]), w[j + F - 1]);
#pragma unroll
        for (int q = 2; q <= F; ++q) {
          da = f2fma(dup2(A.ct1[q]), w[j + F + q], da);
          db = f2fma(dup2(-A.ct1[q]), w[j + F - q], db);
        }
        const float2 d = f2add(da, db);
        vth[j] = zw ? cmulf(d, pz) : d;
      }
    }
    float2 done[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) done[j] = forward_row<HEL>(acc[j], xv[j], inp[j], vth[j], is_out, A.cz2, A.cz1);
    if (it >= 2 * F) {                     // output plane zo = zi - F is complete
      const int zo = zi - F;
      const float2* xp_t = (const float2*)(oring + (size_t)os * A.ostage_bytes);
      if (A.use_xprev) {
        ocur = it - 2 * F;
        if (!mbar_wait_bounded(&ofull[os], (uint32_t)opar)) failed = true;
        ocur = it - 2 * F + 1;
      }
#pragma unroll
      for (int j = 0; j < RPT; ++j) {
        const int t = wy * RPT + j;
        if (rok && t < TY) {
          // out = alpha (Veff x - lap/2 - c x) + beta xprev = -alpha/2 acc + beta xprev
          float2 o = f2mul(mhalf_alpha, done[j]);
          if (A.use_xprev) o = f2fma(dup2(beta), xp_t[t * 32 + lane], o);
          out[(size_t)zo * plane + (size_t)(t0 + t) * Nx + r] = o;
        }
      }
      if (A.use_xprev && ++os == NOS) { os = 0; opar ^= 1; }
    }
    if (__syncthreads_or(failed)) failed = true;
    if (!failed && threadIdx.x == 0) {
      // halo rows were written through the generic proxy before the stage is refilled by TMA
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (issued < nplanes) { issue_x(issued); ++issued; }
      if (A.use_xprev && it >= 2 * F && oissued < nout) { issue_o(oissued); ++oissued; }
    }
    s = s1;
    par = par1;
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicExch(A.status, 1);
      // drain this CTA's copies that were issued but not awaited before its shared memory is
      // released (bounded waits)
      for (int it = waited; it < issued; ++it) mbar_wait_bounded(&full[it % NST], (uint32_t)((it / NST) & 1));
      for (int io = ocur; io < oissued; ++io) mbar_wait_bounded(&ofull[io % NOS], (uint32_t)((io / NOS) & 1));
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------- host side
static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  // looked up once (thread-safe static initialisation)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)p;
    return nullptr;
  }();
  return fn;
}

struct TileGeom {
  int TY, tiles_t, rpt, warps, stage_bytes, nst, ostage_bytes, nos;
};

static size_t tma_smem_bytes(const TileGeom& t) {
  return 256 + (size_t)t.nst * t.stage_bytes + (size_t)t.nos * t.ostage_bytes;
}

// Theta tiling: one tile of all Ny rows when Ny <= 24 (helical cells: <= 36), else the fewest
// equal tiles of <= 24 rows.  Tile rows must be a multiple of 4 so that every staged row block
// starts on a 128-byte boundary (row pitch 352 B), and >= the 8-row halo.
// rpt (rows per thread) and prefetch depth: the given ones when valid (rpt > 0, p > 0), else
// the default rule: the fewest rows per thread with at most 12 warps, the deepest prefetch that fits.
static bool tile_geometry(const GridDev& g, TileGeom* t, int rpt = 0, int p_req = 0) {
  // (z wraps at most once: Nz >= FDn)
  if (g.FDn != TM_F || g.BCy != 0 || g.Ny < TM_HALO || g.Nz < TM_F) return false;
  int ty = 0, nt = 0;
  if (g.helical) {
    if (g.Ny <= 36 && g.Ny % 4 == 0) { ty = g.Ny; nt = 1; }
  } else {
    for (int n = 1; n <= g.Ny; ++n)
      if (g.Ny % n == 0 && (g.Ny / n) % 4 == 0 && g.Ny / n <= 24 && g.Ny / n >= TM_HALO) { ty = g.Ny / n; nt = n; break; }
  }
  if (ty == 0) return false;
  t->TY = ty;
  t->tiles_t = nt;
  t->rpt = rpt > 0 ? rpt : (ty + TM_MAXW - 1) / TM_MAXW;
  if (t->rpt < 1 || t->rpt > 3) return false;
  t->warps = (ty + t->rpt - 1) / t->rpt;
  if (t->warps > (t->rpt == 1 ? TM_MAXW1 : TM_MAXW)) return false;
  t->stage_bytes = TM_BW * (ty + 2 * TM_HALO) * 8 + 32 * ty * 4;   // rows + Veff tile
  t->ostage_bytes = 32 * ty * 8;                                    // previous iterate tile
  // the deepest prefetch (P X planes and P xprev tiles in flight) that fits, or the requested one
  for (int p = p_req > 0 ? p_req : TM_PMAX; p >= 2; --p) {
    t->nst = 1 + p;
    t->nos = p;
    if (tma_smem_bytes(*t) <= TM_SMEM_MAX) return true;
    if (p_req > 0) return false;
  }
  return false;
}

// (rows per thread, prefetch depth) candidates of the autotuner for this grid
int tma_candidates(const GridDev& g, int* rpt, int* depth, int cap) {
  // ring depths 2..6 and 8 (odd ones too: at 3 rows per thread a depth of 5 still keeps two CTAs
  // per SM, 6 does not)
  static const int depths[] = {2, 3, 4, 5, 6, 8};
  int n = 0;
  for (int r = 1; r <= 3; ++r)
    for (int p : depths) {
      TileGeom t;
      if (p <= TM_PMAX && n < cap && tile_geometry(g, &t, r, p)) { rpt[n] = r; depth[n] = p; ++n; }
    }
  return n;
}

bool tma_eligible(const GridDev& g, int elem_bytes) {
  if (elem_bytes != 8) return false;                // complex64 only
  if (g.Nx % 4 != 0) return false;                  // row pitches must be multiples of 16 B (float and complex64 maps)
  TileGeom t;
  if (!tile_geometry(g, &t)) return false;
  return get_encode() != nullptr;
}

static cx_status encode(cx_handle h, CUtensorMap* out, CUtensorMapDataType dt, int rank, const void* base, const cuuint64_t* dims,
                        const cuuint64_t* strides, const cuuint32_t* box) {
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUresult r = get_encode()(out, dt, rank, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    h->err = "cuTensorMapEncodeTiled failed with status " + std::to_string((int)r);
    return CX_ERR_CUDA;
  }
  return CX_OK;
}

// Maps of one complex64 buffer holding Ns states: dims (Nr, Ny, Nz, Ns), 8-byte elements.
// xmap: the TY staged rows (box TM_BW x TY); hmap: a theta halo (TM_BW x 8); omap: the output
// tile (32 x TY).
cx_status make_buffer_maps(cx_handle h, const void* base, int Ns, CUtensorMap_st* xmap, CUtensorMap_st* hmap, CUtensorMap_st* omap) {
  const GridDev& g = h->g;
  TileGeom t;
  if (!tile_geometry(g, &t)) { h->err = "tensor maps: grid not eligible for the TMA stencil"; return CX_ERR_ARG; }
  cuuint64_t dims[4] = {(cuuint64_t)g.Nx, (cuuint64_t)g.Ny, (cuuint64_t)g.Nz, (cuuint64_t)Ns};
  cuuint64_t strides[3] = {(cuuint64_t)g.Nx * 8, (cuuint64_t)g.Nx * g.Ny * 8, (cuuint64_t)g.Nx * g.Ny * g.Nz * 8};
  cuuint32_t box[4] = {(cuuint32_t)TM_BW, (cuuint32_t)t.TY, 1, 1};
  cx_status s = encode(h, (CUtensorMap*)xmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, box);
  if (s != CX_OK) return s;
  cuuint32_t hbox[4] = {(cuuint32_t)TM_BW, (cuuint32_t)TM_HALO, 1, 1};
  if ((s = encode(h, (CUtensorMap*)hmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, hbox)) != CX_OK) return s;
  cuuint32_t obox[4] = {32, (cuuint32_t)t.TY, 1, 1};
  return encode(h, (CUtensorMap*)omap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, obox);
}

// Map of a 4-byte scalar grid field (N values): dims (Nr, Ny, Nz), box 32 x TY.
cx_status make_field_map(cx_handle h, const void* base, bool is_int, CUtensorMap_st* out) {
  const GridDev& g = h->g;
  TileGeom t;
  if (!tile_geometry(g, &t)) { h->err = "tensor maps: grid not eligible for the TMA stencil"; return CX_ERR_ARG; }
  cuuint64_t dims[3] = {(cuuint64_t)g.Nx, (cuuint64_t)g.Ny, (cuuint64_t)g.Nz};
  cuuint64_t strides[2] = {(cuuint64_t)g.Nx * 4, (cuuint64_t)g.Nx * g.Ny * 4};
  cuuint32_t box[3] = {32, (cuuint32_t)t.TY, 1};
  return encode(h, (CUtensorMap*)out, is_int ? CU_TENSOR_MAP_DATA_TYPE_INT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims,
                strides, box);
}

template <int RPT, bool HEL>
static cudaError_t launch_tma_inst(const TmaArgs& a, dim3 grid, int threads, size_t smem, cudaStream_t st) {
  auto kern = cheb_tma_kernel<RPT, HEL>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, threads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cheb_step_tma(const GridDev& g, const StencilCoef& coef, const BlockDev<float>* blocks, const StepScalars* scal,
                                 const int2* state_tab, int nstates, int in_sel, bool use_xprev, const TmaMapSet& maps, int* status,
                                 cudaStream_t st, int rpt, int depth) {
  TileGeom t;
  if (!tile_geometry(g, &t, rpt, depth)) return cudaErrorInvalidValue;
  TmaArgs a{};
  a.g = g;
  a.blocks = blocks;
  a.scal = scal;
  a.state_tab = state_tab;
  a.xmaps = (const CUtensorMap*)maps.xmaps;
  a.hmaps = (const CUtensorMap*)maps.hmaps;
  a.omaps = (const CUtensorMap*)maps.omaps;
  a.vmaps = (const CUtensorMap*)maps.vmaps;
  a.status = status;
  a.tiles_r = (g.Nx + TM_TR - 1) / TM_TR;
  a.tiles_t = t.tiles_t;
  a.TY = t.TY;
  a.stage_bytes = t.stage_bytes;
  a.nst = t.nst;
  a.ostage_bytes = t.ostage_bytes;
  a.nos = t.nos;
  // one CTA per SM at a time: whole-z items fill full waves, the remainder is split along z
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
    nsm = 1;
  const long items = (long)a.tiles_r * t.tiles_t * nstates;
  const long rem = items % nsm;
  a.zsplit = 1;
  a.full_items = (int)items;
  if (rem != 0) {
    a.zsplit = (int)std::max(1L, std::min((long)nsm / rem, (long)(g.Nz / 8)));
    a.full_items = (int)(items - rem);
  }
  const long ctas = a.full_items + rem * a.zsplit;
  if (ctas > 0x7fffffffL) return cudaErrorInvalidConfiguration;
  a.in_sel = in_sel;
  a.use_xprev = use_xprev ? 1 : 0;
  for (int q = 0; q <= TM_F; ++q) {
    a.cr2[q] = (float)coef.cr2[q]; a.cr1[q] = (float)coef.cr1[q];
    a.ct2[q] = (float)coef.ct2[q]; a.ct1[q] = (float)coef.ct1[q];
    a.cz2[q] = (float)coef.cz2[q]; a.cz1[q] = (float)coef.cz1[q];
  }
  const int threads = 32 * t.warps;
  const size_t smem = tma_smem_bytes(t);
  dim3 grid((unsigned)ctas, 1);
  switch (t.rpt * 2 + (g.helical ? 1 : 0)) {
    case 2: return launch_tma_inst<1, false>(a, grid, threads, smem, st);
    case 3: return launch_tma_inst<1, true>(a, grid, threads, smem, st);
    case 4: return launch_tma_inst<2, false>(a, grid, threads, smem, st);
    case 5: return launch_tma_inst<2, true>(a, grid, threads, smem, st);
    case 6: return launch_tma_inst<3, false>(a, grid, threads, smem, st);
    case 7: return launch_tma_inst<3, true>(a, grid, threads, smem, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cx
