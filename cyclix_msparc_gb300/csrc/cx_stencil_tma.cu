// TMA-pipelined fused H*psi / Chebyshev step for complex64 blocks (the production path of the
// mixed-precision filter).  Same arithmetic as cheb_step_kernel in cx_stencil.cu
// (Cychel/lapVec_cychel.m:19-52, src/h_nonlocal_vector_mult.m:21-43, src/chebyshev_filter.m:24-42),
// different data movement:
//
//  * a CTA owns TR = 32 radial points x ALL theta rows of one state and marches along z over a
//    chunk of output planes; theta neighbours wrap inside the tile (Bloch phase applied in
//    registers, warp-uniform), so no theta halo is ever re-read;
//  * every z-plane of the tile (+ FDn radial halo, zero-filled by TMA outside [0, Nr): the
//    Dirichlet walls) is copied HBM -> shared memory once by cp.async.bulk.tensor.4d into a ring of
//    NST = FDn + 1 + P stages guarded by mbarriers, P planes ahead of the consumer;
//  * the per-output-plane operands -- the previous Chebyshev iterate and Veff (a float copy) --
//    arrive by TMA in a second, shorter ring, so the output path reads shared memory only;
//  * the Kleinman-Bylander term is not part of this kernel: nl_apply_kernel (cx_stencil.cu) adds it
//    afterwards on the 32-point row chunks that a projector ball touches;
//  * the in-plane (r, theta) part of the stencil of output plane zo is read from the ring; the z
//    neighbourhood of each thread's column lives in a 2*FDn+1 register queue;
//  * helical cells: the cross term (X DG2^T) DG3^T = D_theta(D_z X) is formed by writing D_z X of
//    each thread's rows to a shared-memory row buffer and applying D_theta from there;
//  * mbarrier waits are bounded; on a timeout the CTA records it in *status, drains its own
//    outstanding copies (again bounded) and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "cx_common.h"

namespace cx {

constexpr int TMA_TR = 32;
constexpr int TMA_P = 3;       // X planes prefetched ahead of the consumer
constexpr int TMA_NO = 3;      // stages of the output-operand ring
constexpr int TMA_OAHEAD = 2;  // output planes prefetched ahead

struct TmaArgs {
  GridDev g;
  const BlockDev<float>* blocks;
  const StepScalars* scal;
  const int2* state_tab;
  const CUtensorMap* xmaps;     // [block][buffer], box = staged X tile
  const CUtensorMap* omaps;     // [block][buffer], box = 32 x Ny output tile
  const CUtensorMap* vmaps;     // [spin] float Veff
  int* status;
  int tiles_r, zc, in_sel, use_xprev;
  int bwt, xoff, stage_bytes, nst, ostage_bytes;
  float cr2[kMaxFDn + 1], cr1[kMaxFDn + 1], ct2[kMaxFDn + 1], ct1[kMaxFDn + 1], cz2[kMaxFDn + 1], cz1[kMaxFDn + 1];
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
// bounded wait: true when the phase completed, false after the iteration limit
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); ++i)
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

__device__ __forceinline__ float2 pmulf(float2 v, double2 p) {
  const float px = (float)p.x, py = (float)p.y;
  return make_float2(v.x * px - v.y * py, v.x * py + v.y * px);
}

// F: FDn, RPT: theta rows per thread, HEL: helical cross term
template <int F, int RPT, bool HEL>
__global__ void __launch_bounds__(384, 1) cheb_tma_kernel(const __grid_constant__ TmaArgs A) {
  constexpr int Q = 2 * F + 1;
  extern __shared__ __align__(128) unsigned char smem[];
  const int Nx = A.g.Nx, Ny = A.g.Ny, Nz = A.g.Nz;
  const int NST = A.nst;
  uint64_t* full = (uint64_t*)smem;                                       // NST barriers (X ring)
  uint64_t* ofull = full + 16;                                            // TMA_NO barriers (output ring)
  unsigned char* ring = smem + 256;
  unsigned char* oring = ring + (size_t)NST * A.stage_bytes;
  float2* ubuf = (float2*)(oring + (size_t)TMA_NO * A.ostage_bytes);      // helical: Ny x 32 row buffer
  const int BW = A.bwt;

  const int lane = threadIdx.x & 31;
  const int wy = threadIdx.x >> 5;
  const int gs = blockIdx.y;
  const int2 bs = A.state_tab[gs];
  const BlockDev<float>& B = A.blocks[bs.x];
  const size_t plane = (size_t)Nx * Ny;
  const size_t sN = (size_t)bs.y * plane * Nz;
  float2* __restrict__ out = B.buf[A.in_sel ^ 1] + sN;
  const double2 ph_tl = B.ph_tl, ph_tr = B.ph_tr, ph_zl = B.ph_zl, ph_zr = B.ph_zr;
  const StepScalars sc = A.scal[bs.x];
  const float alpha = (float)sc.alpha, cshift = (float)sc.c, beta = (float)sc.beta;
  const CUtensorMap* xmap = A.xmaps + 2 * bs.x + A.in_sel;
  const CUtensorMap* omap = A.omaps + 2 * bs.x + (A.in_sel ^ 1);
  const CUtensorMap* vmap = A.vmaps + B.veff_spin;
  const bool bcy = A.g.BCy != 0, bcz = A.g.BCz != 0;

  const int ir = blockIdx.x % A.tiles_r;
  const int iz = blockIdx.x / A.tiles_r;
  const int r0 = ir * TMA_TR;
  const int z0 = iz * A.zc;
  const int z1 = min(z0 + A.zc, Nz);
  const int zstart = z0 - F, zend = z1 + F;          // X planes entering the CTA
  const int nplanes = zend - zstart;
  const int nout = z1 - z0;

  const int r = r0 + lane;
  const bool rok = r < Nx;
  const double rr = A.g.xin + (double)r * A.g.dx;
  const float inv_r = (float)(1.0 / rr);
  const float th_scale = HEL ? (float)(A.g.twist * A.g.twist + 1.0 / (rr * rr)) : (float)(1.0 / (rr * rr));
  float cp_[F + 1], cm_[F + 1];
#pragma unroll
  for (int q = 0; q <= F; ++q) {
    cp_[q] = A.cr2[q] + inv_r * A.cr1[q];
    cm_[q] = A.cr2[q] - inv_r * A.cr1[q];
  }
  const int col = lane + F + A.xoff;
  const int ob_x = 32 * Ny * 8;             // bytes of the xprev tile in an output stage
  const int ob_v = 32 * Ny * 4;             // veff tile
  const uint32_t xbytes = (uint32_t)(BW * Ny * 8);
  const uint32_t obytes = (uint32_t)((A.use_xprev ? ob_x : 0) + ob_v);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) mbar_init(&full[s], 1);
    for (int s = 0; s < TMA_NO; ++s) mbar_init(&ofull[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue_x = [&](int it) {             // X plane zstart + it into stage it % NST
    const int s = it % NST;
    int zc = zstart + it;
    if (!bcz) { if (zc < 0) zc += Nz; else if (zc >= Nz) zc -= Nz; }
    mbar_expect_tx(&full[s], xbytes);
    tma_load_4d(ring + (size_t)s * A.stage_bytes, xmap, &full[s], r0 - F - A.xoff, 0, zc, bs.y);
  };
  auto issue_o = [&](int io) {             // output operands of plane z0 + io into stage io % TMA_NO
    const int s = io % TMA_NO;
    const int zo = z0 + io;
    unsigned char* dst = oring + (size_t)s * A.ostage_bytes;
    mbar_expect_tx(&ofull[s], obytes);
    if (A.use_xprev) tma_load_4d(dst, omap, &ofull[s], r0, 0, zo, bs.y);
    tma_load_3d(dst + ob_x, vmap, &ofull[s], r0, 0, zo);
  };
  int issued = 0, oissued = 0;
  if (threadIdx.x == 0) {
    const int n0 = min(NST, nplanes);
    for (int k = 0; k < n0; ++k) issue_x(k);
    issued = n0;
    const int m0 = min(TMA_OAHEAD + 1, nout);
    for (int k = 0; k < m0; ++k) issue_o(k);
    oissued = m0;
  }

  float2 zq[RPT][Q];
#pragma unroll
  for (int j = 0; j < RPT; ++j)
#pragma unroll
    for (int k = 0; k < Q; ++k) zq[j][k] = make_float2(0.f, 0.f);

  const bool wfast = (wy * RPT - F >= 0) && (wy * RPT + RPT - 1 + F <= Ny - 1);   // window does not wrap
  bool failed = false;
  int cur = 0, ocur = 0;
  int s = 0, par = 0;                      // X-ring stage and parity of plane `it`
  int os = 0, opar = 0;                    // output-ring stage and parity
  for (int it = 0; it < nplanes; ++it) {
    const int zi = zstart + it;
    cur = it;
    if (!mbar_wait_bounded(&full[s], (uint32_t)par)) failed = true;
    const float2* P = (const float2*)(ring + (size_t)s * A.stage_bytes);
    const bool zw = !bcz && (zi < 0 || zi >= Nz);
    const double2 pz = zi < 0 ? ph_zl : ph_zr;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
#pragma unroll
      for (int k = 0; k < Q - 1; ++k) zq[j][k] = zq[j][k + 1];
      const int t = wy * RPT + j;
      float2 c = t < Ny ? P[(size_t)t * BW + col] : make_float2(0.f, 0.f);
      if (zw) c = pmulf(c, pz);
      zq[j][Q - 1] = c;
    }
    const int zo = zi - F;
    if (zo >= z0) {
      ocur = zo - z0;
      if (!mbar_wait_bounded(&ofull[os], (uint32_t)opar)) failed = true;
      int so = s - F;
      if (so < 0) so += NST;
      const float2* Po = (const float2*)(ring + (size_t)so * A.stage_bytes);
      const unsigned char* ost = oring + (size_t)os * A.ostage_bytes;
      const float2* xp_t = (const float2*)ost;
      const float* v_t = (const float*)(ost + ob_x);
      // theta window of this thread's rows (rows wy*RPT-F .. wy*RPT+RPT-1+F of plane zo)
      float2 win[RPT + 2 * F];
      if (wfast) {
#pragma unroll
        for (int w = 0; w < RPT + 2 * F; ++w) win[w] = Po[(size_t)(wy * RPT + w - F) * BW + col];
      } else {
#pragma unroll
        for (int w = 0; w < RPT + 2 * F; ++w) {
          int t = wy * RPT + w - F;
          float2 v;
          if (t < 0) {
            t += Ny;
            v = bcy ? make_float2(0.f, 0.f) : pmulf(Po[(size_t)t * BW + col], ph_tl);
          } else if (t >= Ny) {
            t -= Ny;
            v = (bcy || t >= Ny) ? make_float2(0.f, 0.f) : pmulf(Po[(size_t)t * BW + col], ph_tr);
          } else {
            v = Po[(size_t)t * BW + col];
          }
          win[w] = v;
        }
      }
      float2 lapv[RPT];
#pragma unroll
      for (int j = 0; j < RPT; ++j) {
        const int t = wy * RPT + j;
        const float2* row = Po + (size_t)(t < Ny ? t : 0) * BW;
        const float2 x0 = zq[j][F];
        float2 lap = make_float2(cp_[0] * x0.x, cp_[0] * x0.y);
#pragma unroll
        for (int q = 1; q <= F; ++q) {
          const float2 a = row[col + q], b = row[col - q];
          lap.x = fmaf(cp_[q], a.x, lap.x); lap.y = fmaf(cp_[q], a.y, lap.y);
          lap.x = fmaf(cm_[q], b.x, lap.x); lap.y = fmaf(cm_[q], b.y, lap.y);
        }
        float2 st2 = make_float2(A.ct2[0] * win[j + F].x, A.ct2[0] * win[j + F].y);
#pragma unroll
        for (int q = 1; q <= F; ++q) {
          st2.x = fmaf(A.ct2[q], win[j + F + q].x + win[j + F - q].x, st2.x);
          st2.y = fmaf(A.ct2[q], win[j + F + q].y + win[j + F - q].y, st2.y);
        }
        lap.x = fmaf(th_scale, st2.x, lap.x); lap.y = fmaf(th_scale, st2.y, lap.y);
        lap.x = fmaf(A.cz2[0], x0.x, lap.x); lap.y = fmaf(A.cz2[0], x0.y, lap.y);
#pragma unroll
        for (int q = 1; q <= F; ++q) {
          lap.x = fmaf(A.cz2[q], zq[j][F + q].x + zq[j][F - q].x, lap.x);
          lap.y = fmaf(A.cz2[q], zq[j][F + q].y + zq[j][F - q].y, lap.y);
        }
        lapv[j] = lap;
      }
      if (HEL) {
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
          float2 u = make_float2(0.f, 0.f);
#pragma unroll
          for (int q = 1; q <= F; ++q) {
            u.x = fmaf(A.cz1[q], zq[j][F + q].x - zq[j][F - q].x, u.x);
            u.y = fmaf(A.cz1[q], zq[j][F + q].y - zq[j][F - q].y, u.y);
          }
          const int t = wy * RPT + j;
          if (t < Ny) ubuf[(size_t)t * 32 + lane] = u;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
          const int t = wy * RPT + j;
          float2 cr = make_float2(0.f, 0.f);
#pragma unroll
          for (int q = 1; q <= F; ++q) {
            int tp = t + q, tm = t - q;
            float2 a, b;
            if (tp >= Ny) { tp -= Ny; a = (bcy || tp >= Ny) ? make_float2(0.f, 0.f) : pmulf(ubuf[(size_t)tp * 32 + lane], ph_tr); }
            else a = ubuf[(size_t)tp * 32 + lane];
            if (tm < 0) { tm += Ny; b = (bcy || tm < 0) ? make_float2(0.f, 0.f) : pmulf(ubuf[(size_t)tm * 32 + lane], ph_tl); }
            else b = ubuf[(size_t)tm * 32 + lane];
            cr.x = fmaf(A.ct1[q], a.x - b.x, cr.x);
            cr.y = fmaf(A.ct1[q], a.y - b.y, cr.y);
          }
          lapv[j].x += cr.x;
          lapv[j].y += cr.y;
        }
      }
#pragma unroll
      for (int j = 0; j < RPT; ++j) {
        const int t = wy * RPT + j;
        if (rok && t < Ny) {
          const int li = t * 32 + lane;
          const float2 x0 = zq[j][F];
          const float v = v_t[li];
          const float2 hy = make_float2(fmaf(v, x0.x, -0.5f * lapv[j].x), fmaf(v, x0.y, -0.5f * lapv[j].y));
          float2 o = make_float2(alpha * (hy.x - cshift * x0.x), alpha * (hy.y - cshift * x0.y));
          if (A.use_xprev) {
            const float2 xp = xp_t[li];
            o.x = fmaf(beta, xp.x, o.x);
            o.y = fmaf(beta, xp.y, o.y);
          }
          out[(size_t)zo * plane + (size_t)t * Nx + r] = o;
        }
      }
      if (++os == TMA_NO) { os = 0; opar ^= 1; }
    }
    // every thread is done with plane zo, its output operands and ubuf: recycle the stages
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    if (threadIdx.x == 0) {
      if (zo >= zstart && issued < nplanes) { issue_x(issued); ++issued; }
      if (zo >= z0 && oissued < nout) { issue_o(oissued); ++oissued; }
    }
    if (++s == NST) { s = 0; par ^= 1; }
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicExch(A.status, 1);
      // drain this CTA's copies that were issued but not consumed before its shared memory is
      // released (bounded waits)
      for (int it = cur; it < issued; ++it) mbar_wait_bounded(&full[it % NST], (uint32_t)((it / NST) & 1));
      for (int io = ocur; io < oissued; ++io) mbar_wait_bounded(&ofull[io % TMA_NO], (uint32_t)((io / TMA_NO) & 1));
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------- host side
static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

int tma_rows_per_thread(int Ny) {
  for (int rpt = 1; rpt <= 4; ++rpt)
    if ((Ny + rpt - 1) / rpt <= 12) return rpt;
  return 0;
}

static void tma_tile_geometry(const GridDev& g, int* bwt, int* xoff, int* stage_bytes, int* nst, int* ostage_bytes) {
  const int F = g.FDn;
  *xoff = (F & 1);                                  // start column rounded down to an even index
  *bwt = TMA_TR + 2 * F + 2 * (F & 1);
  *stage_bytes = ((*bwt * g.Ny * 8) + 127) / 128 * 128;
  *nst = F + 1 + TMA_P;
  *ostage_bytes = ((32 * g.Ny * (8 + 4)) + 127) / 128 * 128;
}

static size_t tma_smem_bytes(const GridDev& g) {
  int bwt, xoff, sb, nst, osb;
  tma_tile_geometry(g, &bwt, &xoff, &sb, &nst, &osb);
  return 256 + (size_t)nst * sb + (size_t)TMA_NO * osb + (g.helical ? (size_t)g.Ny * 32 * 8 : 0);
}

bool tma_eligible(const GridDev& g, int elem_bytes) {
  if (elem_bytes != 8) return false;                // complex64 only
  if (g.FDn != 6) return false;                     // instantiated for FD order 12
  if (g.Nx % 4 != 0) return false;                  // row pitches must be multiples of 16 B (float and complex64 maps)
  if (tma_rows_per_thread(g.Ny) == 0) return false;
  if (tma_smem_bytes(g) > 227 * 1024) return false;
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
// xmap: box of the staged X tile (bwt x Ny); omap: box of the output tile (32 x Ny).
cx_status make_buffer_maps(cx_handle h, const void* base, int Ns, CUtensorMap_st* xmap, CUtensorMap_st* omap) {
  const GridDev& g = h->g;
  int bwt, xoff, sb, nst, osb;
  tma_tile_geometry(g, &bwt, &xoff, &sb, &nst, &osb);
  cuuint64_t dims[4] = {(cuuint64_t)g.Nx, (cuuint64_t)g.Ny, (cuuint64_t)g.Nz, (cuuint64_t)Ns};
  cuuint64_t strides[3] = {(cuuint64_t)g.Nx * 8, (cuuint64_t)g.Nx * g.Ny * 8, (cuuint64_t)g.Nx * g.Ny * g.Nz * 8};
  cuuint32_t box[4] = {(cuuint32_t)bwt, (cuuint32_t)g.Ny, 1, 1};
  cx_status s = encode(h, (CUtensorMap*)xmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, box);
  if (s != CX_OK) return s;
  cuuint32_t obox[4] = {32, (cuuint32_t)g.Ny, 1, 1};
  return encode(h, (CUtensorMap*)omap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, obox);
}

// Map of a 4-byte scalar grid field (N values): dims (Nr, Ny, Nz), box 32 x Ny.
cx_status make_field_map(cx_handle h, const void* base, bool is_int, CUtensorMap_st* out) {
  const GridDev& g = h->g;
  cuuint64_t dims[3] = {(cuuint64_t)g.Nx, (cuuint64_t)g.Ny, (cuuint64_t)g.Nz};
  cuuint64_t strides[2] = {(cuuint64_t)g.Nx * 4, (cuuint64_t)g.Nx * g.Ny * 4};
  cuuint32_t box[3] = {32, (cuuint32_t)g.Ny, 1};
  return encode(h, (CUtensorMap*)out, is_int ? CU_TENSOR_MAP_DATA_TYPE_INT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims,
                strides, box);
}

template <int F, int RPT, bool HEL>
static cudaError_t launch_tma_inst(const TmaArgs& a, dim3 grid, int threads, size_t smem, cudaStream_t st) {
  auto kern = cheb_tma_kernel<F, RPT, HEL>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, threads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cheb_step_tma(const GridDev& g, const StencilCoef& coef, const BlockDev<float>* blocks, const StepScalars* scal,
                                 const int2* state_tab, int nstates, int in_sel, bool use_xprev, const TmaMapSet& maps, int* status,
                                 cudaStream_t st) {
  TmaArgs a{};
  a.g = g;
  a.blocks = blocks;
  a.scal = scal;
  a.state_tab = state_tab;
  a.xmaps = (const CUtensorMap*)maps.xmaps;
  a.omaps = (const CUtensorMap*)maps.omaps;
  a.vmaps = (const CUtensorMap*)maps.vmaps;
  a.status = status;
  a.tiles_r = (g.Nx + TMA_TR - 1) / TMA_TR;
  tma_tile_geometry(g, &a.bwt, &a.xoff, &a.stage_bytes, &a.nst, &a.ostage_bytes);
  const long ctas = (long)a.tiles_r * nstates;
  int nzc = 1;
  while (ctas * nzc < 2 * 152 && g.Nz / (nzc * 2) >= 8) nzc *= 2;
  a.zc = (g.Nz + nzc - 1) / nzc;
  const int zchunks = (g.Nz + a.zc - 1) / a.zc;
  a.in_sel = in_sel;
  a.use_xprev = use_xprev ? 1 : 0;
  for (int q = 0; q <= kMaxFDn; ++q) {
    a.cr2[q] = (float)coef.cr2[q]; a.cr1[q] = (float)coef.cr1[q];
    a.ct2[q] = (float)coef.ct2[q]; a.ct1[q] = (float)coef.ct1[q];
    a.cz2[q] = (float)coef.cz2[q]; a.cz1[q] = (float)coef.cz1[q];
  }
  if (nstates > 65535) return cudaErrorInvalidConfiguration;
  const int rpt = tma_rows_per_thread(g.Ny);
  const int threads = 32 * ((g.Ny + rpt - 1) / rpt);
  const size_t smem = tma_smem_bytes(g);
  dim3 grid((unsigned)(a.tiles_r * zchunks), (unsigned)nstates);
  if (g.FDn != 6) return cudaErrorInvalidValue;
  switch (rpt * 2 + (g.helical ? 1 : 0)) {
    case 2: return launch_tma_inst<6, 1, false>(a, grid, threads, smem, st);
    case 3: return launch_tma_inst<6, 1, true>(a, grid, threads, smem, st);
    case 4: return launch_tma_inst<6, 2, false>(a, grid, threads, smem, st);
    case 5: return launch_tma_inst<6, 2, true>(a, grid, threads, smem, st);
    case 6: return launch_tma_inst<6, 3, false>(a, grid, threads, smem, st);
    case 7: return launch_tma_inst<6, 3, true>(a, grid, threads, smem, st);
    case 8: return launch_tma_inst<6, 4, false>(a, grid, threads, smem, st);
    case 9: return launch_tma_inst<6, 4, true>(a, grid, threads, smem, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cx
