// Fused Hamiltonian application and Chebyshev three-term step on the Cyclix grid.
//
// One launch applies, to every state of every Bloch block at once,
//     out = alpha * (H*in - c*in) + beta * xprev,
//     H*in = -1/2 Lap(in) + Veff .* in + sum_J Chi_J gamma_J Chi_J^H W in       (per block)
// which is one step of the scaled Chebyshev recurrence of src/chebyshev_filter.m:24-42
// (alpha = 2 sigma2/e, beta = -sigma sigma2; the first step has beta = 0) and, with
// alpha = 1, c = 0, beta = 0, the plain product of src/h_nonlocal_vector_mult.m:21-43.
//
// Lap is the matrix-free form of Cychel/lapVec_cychel.m:19-52:
//   cyclic  (cell_typ 3): (DL11 + DG1) X + R2inv X DL22^T + X DL33^T
//   helical (cell_typ 4/5): adds X DL22^T (tau^2 scaled) and (X DG2^T) DG3^T
// with the 1-D stencils of Cychel/lapIndicesValues_1d_cychel.m (Dirichlet r: out-of-range
// neighbours are zero; theta / z wrap with the Bloch phases of src/blochLaplacian_1d.m:13-37).
//
// Work decomposition: a CTA owns a 32 (r) x 8 (theta) tile of one state and marches along z.
// Each z-plane of the tile plus an FDn-wide r/theta halo is staged in shared memory once
// (double buffered, boundary conditions and Bloch phases applied while staging); each thread
// owns one (r, theta) column and keeps the z-neighbourhood in register queues, so each input
// value is read from HBM once per launch (halo re-reads hit L2).  The in-plane part of the
// Laplacian is evaluated when a plane arrives and delayed FDn planes in registers until the
// z-part of the same output plane is complete.
#include "cx_internal.h"

namespace cx {

constexpr int TR = 32;   // tile extent along r (threads along r; coalesced)
constexpr int TT = 8;    // tile extent along theta
constexpr int NTHR = TR * TT;

template <typename R>
struct StepArgs {
  GridDev g;
  const BlockDev<R>* blocks;
  const StepScalars* scal;      // per block, this degree
  const int2* state_tab;        // global state -> (block, local state)
  int tiles_r, tiles_t, zc;     // tiling
  int in_sel;                   // buffer holding the input of this step
  int use_xprev;
  // nonlocal apply (entries per grid point)
  const int32_t* row_ptr;
  const int32_t* ent_seg;
  const R* ent_chi;
  const cplx<R>* cprime;        // [global state][seg][kAngMax]
  int nseg;
  int nl_on;
  R cr2[kMaxFDn + 1], cr1[kMaxFDn + 1], ct2[kMaxFDn + 1], ct1[kMaxFDn + 1], cz2[kMaxFDn + 1], cz1[kMaxFDn + 1];
};

template <typename R>
__device__ __forceinline__ cplx<R> phase_mul(cplx<R> v, double2 p) {
  cplx<R> o;
  o.x = v.x * (R)p.x - v.y * (R)p.y;
  o.y = v.x * (R)p.y + v.y * (R)p.x;
  return o;
}

template <typename R, int F, bool HEL>
__global__ void __launch_bounds__(NTHR)
cheb_step_kernel(const StepArgs<R> A) {
  constexpr int TW = TR + 2 * F;
  constexpr int TH = TT + 2 * F;
  __shared__ cplx<R> tile[2][TH][TW];

  const int Nx = A.g.Nx, Ny = A.g.Ny, Nz = A.g.Nz;
  const size_t plane = (size_t)Nx * Ny;
  const int tid = threadIdx.x;
  const int tr = tid % TR, tt = tid / TR;

  const int gs = blockIdx.y;
  const int2 bs = A.state_tab[gs];
  const BlockDev<R>& B = A.blocks[bs.x];
  const size_t sN = (size_t)bs.y * plane * Nz;
  const cplx<R>* __restrict__ in = B.buf[A.in_sel] + sN;
  cplx<R>* __restrict__ out = B.buf[A.in_sel ^ 1] + sN;
  const double* __restrict__ veff = B.veff;
  const double2 ph_tl = B.ph_tl, ph_tr = B.ph_tr, ph_zl = B.ph_zl, ph_zr = B.ph_zr;
  const StepScalars sc = A.scal[bs.x];
  const R alpha = (R)sc.alpha, cshift = (R)sc.c, beta = (R)sc.beta;

  int bx = blockIdx.x;
  const int ir = bx % A.tiles_r; bx /= A.tiles_r;
  const int it = bx % A.tiles_t;
  const int iz = bx / A.tiles_t;
  const int r0 = ir * TR, t0 = it * TT;
  const int z0 = iz * A.zc;
  const int z1 = min(z0 + A.zc, Nz);

  const int r = r0 + tr, t = t0 + tt;
  const bool own = (r < Nx) && (t < Ny);
  const double rr = A.g.xin + (double)r * A.g.dx;
  const R inv_r = (R)(1.0 / rr);
  const R th_scale = HEL ? (R)(A.g.twist * A.g.twist + 1.0 / (rr * rr)) : (R)(1.0 / (rr * rr));
  const bool bcy = A.g.BCy != 0, bcz = A.g.BCz != 0;

  cplx<R> zq[2 * F + 1];
  cplx<R> pq[F + 1];
  cplx<R> tq[HEL ? 2 * F + 1 : 1];
  const cplx<R> zero = mk<R>((R)0, (R)0);
#pragma unroll
  for (int i = 0; i < 2 * F + 1; ++i) zq[i] = zero;
#pragma unroll
  for (int i = 0; i < F + 1; ++i) pq[i] = zero;
#pragma unroll
  for (int i = 0; i < (HEL ? 2 * F + 1 : 1); ++i) tq[i] = zero;

  int buf = 0;
  for (int zi = z0 - F; zi < z1 + F; ++zi) {
    // ---- stage plane zi (+ r/theta halo) with boundary conditions and Bloch phases
    {
      int zs = zi;
      double2 pz = make_double2(1.0, 0.0);
      bool zwrap = false, zzero = false;
      if (zi < 0) { if (bcz) zzero = true; else { zs += Nz; pz = ph_zl; zwrap = true; } }
      else if (zi >= Nz) { if (bcz) zzero = true; else { zs -= Nz; pz = ph_zr; zwrap = true; } }
      const cplx<R>* src = in + (size_t)zs * plane;
      for (int idx = tid; idx < TW * TH; idx += NTHR) {
        const int lr = idx % TW, lt = idx / TW;
        const int rg = r0 + lr - F;
        int tg = t0 + lt - F;
        cplx<R> v = zero;
        if (!zzero && rg >= 0 && rg < Nx) {
          bool ok = true, wrap = zwrap;
          double2 p = pz;
          if (tg < 0) {
            if (bcy) ok = false; else { tg += Ny; wrap = true; p = make_double2(p.x * ph_tl.x - p.y * ph_tl.y, p.x * ph_tl.y + p.y * ph_tl.x); }
          } else if (tg >= Ny) {
            if (bcy) ok = false; else { tg -= Ny; wrap = true; p = make_double2(p.x * ph_tr.x - p.y * ph_tr.y, p.x * ph_tr.y + p.y * ph_tr.x); }
          }
          if (tg < 0 || tg >= Ny) ok = false;   // only reached by non-output overhang of tiny grids
          if (ok) {
            v = src[(size_t)tg * Nx + rg];
            if (wrap) v = phase_mul<R>(v, p);
          }
        }
        tile[buf][lt][lr] = v;
      }
    }
    __syncthreads();

    // ---- in-plane part of the Laplacian for plane zi at this thread's column
    const cplx<R>* row = &tile[buf][tt + F][0];
    const cplx<R> xc = row[tr + F];
    cplx<R> s2 = mk<R>(A.cr2[0] * xc.x, A.cr2[0] * xc.y);
    cplx<R> s1 = zero;
    cplx<R> st2 = mk<R>(A.ct2[0] * xc.x, A.ct2[0] * xc.y);
    cplx<R> st1 = zero;
#pragma unroll
    for (int q = 1; q <= F; ++q) {
      const cplx<R> a = row[tr + F + q], b = row[tr + F - q];
      cfma(s2, A.cr2[q], cadd(a, b));
      cfma(s1, A.cr1[q], csub(a, b));
      const cplx<R> c = tile[buf][tt + F + q][tr + F], d = tile[buf][tt + F - q][tr + F];
      cfma(st2, A.ct2[q], cadd(c, d));
      if (HEL) cfma(st1, A.ct1[q], csub(c, d));
    }
    cplx<R> pnew = s2;
    cfma(pnew, inv_r, s1);
    cfma(pnew, th_scale, st2);

#pragma unroll
    for (int i = 0; i < 2 * F; ++i) zq[i] = zq[i + 1];
    zq[2 * F] = xc;
#pragma unroll
    for (int i = 0; i < F; ++i) pq[i] = pq[i + 1];
    pq[F] = pnew;
    if (HEL) {
#pragma unroll
      for (int i = 0; i < 2 * F; ++i) tq[i] = tq[i + 1];
      tq[2 * F] = st1;
    }

    // ---- complete output plane zo = zi - F
    const int zo = zi - F;
    if (zo >= z0 && own) {
      cplx<R> lap = pq[0];
      cfma(lap, A.cz2[0], zq[F]);
#pragma unroll
      for (int q = 1; q <= F; ++q) {
        cfma(lap, A.cz2[q], cadd(zq[F + q], zq[F - q]));
        if (HEL) cfma(lap, A.cz1[q], csub(tq[F + q], tq[F - q]));
      }
      const size_t p = (size_t)zo * plane + (size_t)t * Nx + r;
      const R v = (R)veff[p];
      const cplx<R> x0 = zq[F];
      cplx<R> hy = mk<R>(fma(v, x0.x, (R)-0.5 * lap.x), fma(v, x0.y, (R)-0.5 * lap.y));
      if (A.nl_on) {
        const int e0 = A.row_ptr[p], e1 = A.row_ptr[p + 1];
        const cplx<R>* cp = A.cprime + (size_t)gs * A.nseg * kAngMax;
        for (int e = e0; e < e1; ++e) {
          const cplx<R>* cs = cp + (size_t)A.ent_seg[e] * kAngMax;
          const R* ch = A.ent_chi + (size_t)e * kAngMax;
#pragma unroll
          for (int q = 0; q < kAngMax; ++q) cfma(hy, ch[q], cs[q]);
        }
      }
      cplx<R> o = mk<R>(alpha * (hy.x - cshift * x0.x), alpha * (hy.y - cshift * x0.y));
      if (A.use_xprev) {
        const cplx<R> xp = out[p];
        o.x = fma(beta, xp.x, o.x);
        o.y = fma(beta, xp.y, o.y);
      }
      out[p] = o;
    }
    buf ^= 1;
  }
}

// Contraction of the KB projectors with the block: for atom J and state s,
//   C[J,q,s] = gamma_Jq * sum_img exp(i k.(R_J - R_img)) * sum_n (W Chi_img)[n,q] * in[pos_n, s]
// and the per-image scatter coefficients Cp[s][img][q] = exp(-i k.(R_J - R_img)) C[J,q,s]
// (src/h_nonlocal_vector_mult.m:30-43).  One CTA per (atom, NC_SPC states): the threads walk the
// atom's ball nodes (consecutive along r, so each state's loads coalesce) and read a node's data
// (position, segment, W Chi) once for the NC_SPC states; no atomics.
constexpr int NC_SPC = 4;
template <typename R>
__global__ void __launch_bounds__(128)
nl_contract_kernel(const int N, const int nstates, const BlockDev<R>* __restrict__ blocks, const int2* __restrict__ state_tab,
                   const int in_sel, const NonlocalDev nl, const R* __restrict__ node_wchi, cplx<R>* __restrict__ cprime) {
  const int J = blockIdx.x;
  const int gs0 = blockIdx.y * NC_SPC;
  const int nst = min(NC_SPC, nstates - gs0);
  const cplx<R>* y[NC_SPC];
  const double2* ph[NC_SPC];
  const float2* ph32[NC_SPC];
  // complex64 path: float phases (a double->float conversion per node and state costs more than
  // the loads on GB300's narrow FP64 pipe)
  const bool f32ph = sizeof(R) == 4 && nl.seg_phase32 != nullptr;
#pragma unroll
  for (int j = 0; j < NC_SPC; ++j) {
    const int2 bs = state_tab[gs0 + (j < nst ? j : 0)];
    y[j] = blocks[bs.x].buf[in_sel] + (size_t)bs.y * N;
    ph[j] = nl.seg_phase + (size_t)bs.x * nl.nseg;
    ph32[j] = f32ph ? nl.seg_phase32 + (size_t)bs.x * nl.nseg : nullptr;
  }
  const int n0 = nl.atom_node_ptr[J], n1 = nl.atom_node_ptr[J + 1];
  R a[NC_SPC][2 * kAngMax];
#pragma unroll
  for (int j = 0; j < NC_SPC; ++j)
#pragma unroll
    for (int q = 0; q < 2 * kAngMax; ++q) a[j][q] = 0;
#pragma unroll 2
  for (int n = n0 + threadIdx.x; n < n1; n += blockDim.x) {
    const int pos = nl.node_pos[n];
    const int sg = nl.node_seg[n];
    R wq[kAngMax];
#pragma unroll
    for (int q = 0; q < kAngMax; ++q) wq[q] = node_wchi[(size_t)n * kAngMax + q];
#pragma unroll
    for (int j = 0; j < NC_SPC; ++j) {
      if (j < nst) {
        const cplx<R> v = y[j][pos];
        R px, py;
        if (f32ph) {
          const float2 p = ph32[j][sg];
          px = (R)p.x;
          py = (R)p.y;
        } else {
          const double2 p = ph[j][sg];
          px = (R)p.x;
          py = (R)p.y;
        }
        const R vx = v.x * px - v.y * py;
        const R vy = v.x * py + v.y * px;
#pragma unroll
        for (int q = 0; q < kAngMax; ++q) {
          a[j][2 * q] = fma(wq[q], vx, a[j][2 * q]);
          a[j][2 * q + 1] = fma(wq[q], vy, a[j][2 * q + 1]);
        }
      }
    }
  }
  // CTA reduction: warps by shuffles, then across warps in shared memory
  constexpr int NV = NC_SPC * 2 * kAngMax;
  __shared__ R red[4][NV];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NC_SPC; ++j)
#pragma unroll
    for (int q = 0; q < 2 * kAngMax; ++q) {
      R v = a[j][q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[w][j * 2 * kAngMax + q] = v;
    }
  __syncthreads();
  // threads (state j, segment, q) write the scaled, re-phased coefficients: conj(p) gamma C
  const int s0 = nl.atom_seg_ptr[J], s1 = nl.atom_seg_ptr[J + 1];
  const int nout = nst * (s1 - s0) * kAngMax;
  const int nw = blockDim.x >> 5;
  for (int o = threadIdx.x; o < nout; o += blockDim.x) {
    const int q = o % kAngMax, sg = s0 + (o / kAngMax) % (s1 - s0), j = o / (kAngMax * (s1 - s0));
    R sx = 0, sy = 0;
    for (int k = 0; k < nw; ++k) {
      sx += red[k][j * 2 * kAngMax + 2 * q];
      sy += red[k][j * 2 * kAngMax + 2 * q + 1];
    }
    const R gmm = (R)nl.gamma[(size_t)J * kAngMax + q];
    sx *= gmm;
    sy *= gmm;
    const double2 p = nl.seg_phase[(size_t)state_tab[gs0 + j].x * nl.nseg + sg];
    cplx<R> out;
    out.x = sx * (R)p.x + sy * (R)p.y;
    out.y = sy * (R)p.x - sx * (R)p.y;
    cprime[((size_t)(gs0 + j) * nl.nseg + sg) * kAngMax + q] = out;
  }
}

// Kleinman-Bylander apply as its own pass (used after the TMA stencil, which leaves it out):
//   out[p, s] += alpha_b * sum_{entries e of p} Chi_e . Cp[s][seg_e][:]
// (the scatter of src/h_nonlocal_vector_mult.m:38-42, scaled like the rest of the Chebyshev step).
// Per 32-point row chunk that projector balls touch, the entries form a small dense matrix
// Chi_c (32 points x K = 4 x segments of the chunk, zero where a point is outside a ball), so the
// apply is Y[chunk, states] += Chi_c . Cp_c[K, states]: a CTA owns one chunk and 32 states, stages
// Cp_c of its states in shared memory, and each warp accumulates 4 states for its 32 points with
// coalesced Chi_c loads and broadcast shared-memory reads.
constexpr int NA_SPW = 4;      // states per warp
constexpr int NA_SPC = 8 * NA_SPW;

template <typename R>
__global__ void __launch_bounds__(256)
nl_apply_kernel(const int N, const int Nx, const BlockDev<R>* __restrict__ blocks, const StepScalars* __restrict__ scal,
                const int2* __restrict__ state_tab, const int nstates, const int out_sel, const ChunkTables ct,
                const cplx<R>* __restrict__ cprime, const int nseg) {
  extern __shared__ __align__(16) unsigned char nl_smem[];
  cplx<R>* cs = (cplx<R>*)nl_smem;                       // [NA_SPC][K]
  const int c = blockIdx.x;
  const int p0 = ct.p0[c];
  const int sb = ct.seg_ptr[c], nsc = ct.seg_ptr[c + 1] - sb;
  const int K = nsc * kAngMax;
  const int gsb = blockIdx.y * NA_SPC;
  const int nst_cta = min(NA_SPC, nstates - gsb);
  for (int i = threadIdx.x; i < nst_cta * K; i += blockDim.x) {
    const int sl = i / K, k = i - sl * K;
    const int sg = ct.segs[sb + k / kAngMax];
    cs[i] = cprime[((size_t)(gsb + sl) * nseg + sg) * kAngMax + (k % kAngMax)];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int sl0 = w * NA_SPW;
  if (sl0 >= nst_cta) return;
  const int nst = min(NA_SPW, nst_cta - sl0);
  const int r = p0 % Nx + lane;
  const bool ok = r < Nx;
  const R* __restrict__ chi = (const R*)ct.chi + ct.chi_ptr[c] + lane;     // [K][32]
  cplx<R> acc[NA_SPW];
#pragma unroll
  for (int j = 0; j < NA_SPW; ++j) acc[j] = mk<R>((R)0, (R)0);
  for (int k = 0; k < K; ++k) {
    const R x = chi[(size_t)k * 32];
#pragma unroll
    for (int j = 0; j < NA_SPW; ++j) {
      const cplx<R> v = cs[(sl0 + j) * K + k];
      acc[j].x = fma(x, v.x, acc[j].x);
      acc[j].y = fma(x, v.y, acc[j].y);
    }
  }
  if (!ok) return;
#pragma unroll
  for (int j = 0; j < NA_SPW; ++j) {
    if (j < nst) {
      const int2 bs = state_tab[gsb + sl0 + j];
      const R alpha = (R)scal[bs.x].alpha;
      cplx<R>* out = blocks[bs.x].buf[out_sel] + (size_t)bs.y * N + p0 + lane;
      cplx<R> o = *out;
      o.x = fma(alpha, acc[j].x, o.x);
      o.y = fma(alpha, acc[j].y, o.y);
      *out = o;
    }
  }
}

template <typename R>
cudaError_t launch_nl_apply(const GridDev& g, const BlockDev<R>* blocks, const StepScalars* scal, const int2* state_tab, int nstates,
                            int out_sel, const ChunkTables& ct, const cplx<R>* cprime, int nseg, cudaStream_t st) {
  if (ct.nchunks == 0 || nseg == 0) return cudaSuccess;
  dim3 grid((unsigned)ct.nchunks, (unsigned)((nstates + NA_SPC - 1) / NA_SPC));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  const size_t smem = (size_t)NA_SPC * ct.kmax * sizeof(cplx<R>);
  if (smem > 48 * 1024) {
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(nl_apply_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  nl_apply_kernel<R><<<grid, 256, smem, st>>>(g.N, g.Nx, blocks, scal, state_tab, nstates, out_sel, ct, cprime, nseg);
  return cudaGetLastError();
}

template cudaError_t launch_nl_apply<float>(const GridDev&, const BlockDev<float>*, const StepScalars*, const int2*, int, int,
                                            const ChunkTables&, const cplx<float>*, int, cudaStream_t);
template cudaError_t launch_nl_apply<double>(const GridDev&, const BlockDev<double>*, const StepScalars*, const int2*, int, int,
                                             const ChunkTables&, const cplx<double>*, int, cudaStream_t);

template <typename R, int F, bool HEL>
static cudaError_t launch_one(const StepArgs<R>& a, dim3 grid, cudaStream_t st) {
  cheb_step_kernel<R, F, HEL><<<grid, NTHR, 0, st>>>(a);
  return cudaGetLastError();
}

template <typename R, bool HEL>
static cudaError_t dispatch_fdn(int F, const StepArgs<R>& a, dim3 grid, cudaStream_t st) {
  switch (F) {
    case 1: return launch_one<R, 1, HEL>(a, grid, st);
    case 2: return launch_one<R, 2, HEL>(a, grid, st);
    case 3: return launch_one<R, 3, HEL>(a, grid, st);
    case 4: return launch_one<R, 4, HEL>(a, grid, st);
    case 5: return launch_one<R, 5, HEL>(a, grid, st);
    case 6: return launch_one<R, 6, HEL>(a, grid, st);
    case 7: return launch_one<R, 7, HEL>(a, grid, st);
    case 8: return launch_one<R, 8, HEL>(a, grid, st);
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
cudaError_t launch_cheb_step(const GridDev& g, const StencilCoef& coef, const BlockDev<R>* blocks,
                             const StepScalars* scal, int nblk, const int2* state_tab, int nstates,
                             int in_sel, bool use_xprev, const NonlocalDev* nl, const cplx<R>* cprime,
                             cudaStream_t st) {
  (void)nblk;
  StepArgs<R> a{};
  a.g = g;
  a.blocks = blocks;
  a.scal = scal;
  a.state_tab = state_tab;
  a.tiles_r = (g.Nx + TR - 1) / TR;
  a.tiles_t = (g.Ny + TT - 1) / TT;
  // z-chunk: whole columns unless that leaves too few CTAs to fill the GPU
  const long tiles = (long)a.tiles_r * a.tiles_t * nstates;
  int nzc = 1;
  while (tiles * nzc < 4 * 152 && g.Nz / (nzc * 2) >= 8) nzc *= 2;
  a.zc = (g.Nz + nzc - 1) / nzc;
  const int zchunks = (g.Nz + a.zc - 1) / a.zc;
  a.in_sel = in_sel;
  a.use_xprev = use_xprev ? 1 : 0;
  a.nl_on = (nl && nl->nseg > 0 && cprime) ? 1 : 0;
  if (a.nl_on) {
    a.row_ptr = nl->row_ptr;
    a.ent_seg = nl->ent_seg;
    a.ent_chi = (const R*)nl->ent_chi;
    a.cprime = cprime;
    a.nseg = nl->nseg;
  }
  for (int q = 0; q <= kMaxFDn; ++q) {
    a.cr2[q] = (R)coef.cr2[q]; a.cr1[q] = (R)coef.cr1[q];
    a.ct2[q] = (R)coef.ct2[q]; a.ct1[q] = (R)coef.ct1[q];
    a.cz2[q] = (R)coef.cz2[q]; a.cz1[q] = (R)coef.cz1[q];
  }
  if (nstates > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)(a.tiles_r * a.tiles_t * zchunks), (unsigned)nstates);
  return g.helical ? dispatch_fdn<R, true>(g.FDn, a, grid, st) : dispatch_fdn<R, false>(g.FDn, a, grid, st);
}

template <typename R>
cudaError_t launch_nl_contract(const GridDev& g, const BlockDev<R>* blocks, const int2* state_tab, int nstates,
                               int in_sel, const NonlocalDev& nl, cplx<R>* cprime, cudaStream_t st) {
  if (nl.n_atm == 0 || nl.nseg == 0) return cudaSuccess;
  if (nstates > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)nl.n_atm, (unsigned)((nstates + NC_SPC - 1) / NC_SPC));
  nl_contract_kernel<R><<<grid, 128, 0, st>>>(g.N, nstates, blocks, state_tab, in_sel, nl, (const R*)nl.node_wchi, cprime);
  return cudaGetLastError();
}

template cudaError_t launch_cheb_step<float>(const GridDev&, const StencilCoef&, const BlockDev<float>*, const StepScalars*, int,
                                             const int2*, int, int, bool, const NonlocalDev*, const cplx<float>*, cudaStream_t);
template cudaError_t launch_cheb_step<double>(const GridDev&, const StencilCoef&, const BlockDev<double>*, const StepScalars*, int,
                                              const int2*, int, int, bool, const NonlocalDev*, const cplx<double>*, cudaStream_t);
template cudaError_t launch_nl_contract<float>(const GridDev&, const BlockDev<float>*, const int2*, int, int, const NonlocalDev&,
                                               cplx<float>*, cudaStream_t);
template cudaError_t launch_nl_contract<double>(const GridDev&, const BlockDev<double>*, const int2*, int, int, const NonlocalDev&,
                                                cplx<double>*, cudaStream_t);

}  // namespace cx
