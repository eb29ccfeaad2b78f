// C-ABI entry points of libcyclix_gpu.so: handle lifecycle, operator tables (stencil
// coefficients from Cychel/lapIndicesValues_1d_cychel.m, projector images in the layout of
// calculate_nloc_projector.m), block buffers, host <-> device transfers, H*psi
// (src/h_nonlocal_vector_mult.m) and the Chebyshev filter (src/chebyshev_filter.m).  One
// Chebyshev step on the complex64 path is three launches: projector contraction, TMA stencil,
// projector apply; on the complex128 path two (the apply is fused into the stencil).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <complex>

#include <cuda.h>

#include "cx_internal.h"
#include "cx_common.h"

namespace {
thread_local std::string g_create_err;

template <typename T>
cx_status dalloc(cx_handle h, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    h->err = std::string("cudaMalloc(") + std::to_string(count * sizeof(T)) + " B): " + cudaGetErrorString(e);
    *p = nullptr;
    return CX_ERR_NOMEM;
  }
  return CX_OK;
}

template <typename T>
cx_status upload(cx_handle h, T** p, const std::vector<T>& v) {
  cx_status s = dalloc(h, p, v.size());
  if (s != CX_OK) return s;
  if (!v.empty()) CX_TRY_CUDA(h, cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  h->nl_allocs.push_back((void*)*p);
  return CX_OK;
}

double2 cexp_i(double ang) { return make_double2(std::cos(ang), std::sin(ang)); }

void free_blocks(cx_handle h) {
  for (void* p : h->bufs) cudaFree(p);
  h->bufs.clear();
  for (void* p : h->ubgv) cudaFree(p);
  h->ubgv.clear();
  cudaFree(h->d_blocks); h->d_blocks = nullptr;
  cudaFree(h->d_state_tab); h->d_state_tab = nullptr;
  cudaFree(h->d_cprime); h->d_cprime = nullptr;
  cudaFree(h->d_seg_phase); h->d_seg_phase = nullptr;
  cudaFree(h->d_seg_phase32); h->d_seg_phase32 = nullptr;
  h->nl.seg_phase32 = nullptr;
  cudaFree(h->d_maps); h->d_maps = nullptr;
  h->nl.seg_phase = nullptr;
  h->nblk = 0;
  h->nstates = 0;
  h->blocks.clear();
  h->state0.clear();
}
}  // namespace

namespace cx {

// Device array of BlockDev<R> for the handle's blocks with the given buffer pointers.
template <typename R>
cx_status make_block_devs(cx_handle h, const std::vector<cplx<R>*>& b0, const std::vector<cplx<R>*>& b1,
                          const std::vector<int>& blk_ids, std::vector<BlockDev<R>>& out) {
  out.clear();
  int st = 0;
  for (size_t i = 0; i < blk_ids.size(); ++i) {
    const cx_block& B = h->blocks[blk_ids[i]];
    BlockDev<R> d{};
    d.buf[0] = b0[i];
    d.buf[1] = b1[i];
    d.veff = h->d_veff + (size_t)B.spin * h->g.N;
    const double k2 = B.kpt_vec[1], k3 = B.kpt_vec[2];
    d.ph_tl = k2 == 0 ? make_double2(1, 0) : cexp_i(-k2 * h->grid.L2);
    d.ph_tr = k2 == 0 ? make_double2(1, 0) : cexp_i(k2 * h->grid.L2);
    d.ph_zl = k3 == 0 ? make_double2(1, 0) : cexp_i(-k3 * h->grid.L3);
    d.ph_zr = k3 == 0 ? make_double2(1, 0) : cexp_i(k3 * h->grid.L3);
    d.Ns = B.Ns;
    d.state0 = st;
    d.veff_spin = B.spin;
    st += B.Ns;
    out.push_back(d);
  }
  return CX_OK;
}

// Per-block phases exp(i k.(R_J - R_img)) of every (atom, image) segment (src/h_nonlocal_vector_mult.m:24-28,33).
std::vector<double2> segment_phases(cx_handle h, const cx_block& B) {
  const int nseg = (int)h->seg_atom.size();
  std::vector<double2> ph(nseg);
  const bool gamma = B.kpt_vec[0] == 0 && B.kpt_vec[1] == 0 && B.kpt_vec[2] == 0;
  for (int s = 0; s < nseg; ++s) {
    if (gamma) { ph[s] = make_double2(1, 0); continue; }
    const int J = h->seg_atom[s];
    double dot = 0;
    for (int d = 0; d < 3; ++d) dot += B.kpt_vec[d] * (h->atom_pos[3 * J + d] - h->seg_coord[3 * s + d]);
    ph[s] = cexp_i(dot);
  }
  return ph;
}

// Chebyshev scalars of src/chebyshev_filter.m:19-42 for degrees 1..m.
void cheb_scalars(int m, double a, double b, double a0, std::vector<StepScalars>& out, int stride, int col) {
  const double e = (b - a) / 2, c = (b + a) / 2;
  double sigma = e / (a0 - c);
  const double sigma1 = sigma, gamma = 2 / sigma1;
  out[(size_t)0 * stride + col] = StepScalars{sigma1 / e, c, 0.0, 0.0};
  for (int d = 2; d <= m; ++d) {
    const double sigma2 = 1 / (gamma - sigma);
    out[(size_t)(d - 1) * stride + col] = StepScalars{2 * sigma2 / e, c, -(sigma * sigma2), 0.0};
    sigma = sigma2;
  }
}

// Launch one fused step over the given block set and account profiling.
template <typename R>
cx_status fused_step(cx_handle h, const BlockDev<R>* d_blocks, const StepScalars* d_scal, int nblk, const int2* d_state_tab,
                     int nstates, int in_sel, bool use_xprev, cplx<R>* cprime, bool nonlocal, double bytes, const void* maps) {
  const NonlocalDev* nlp = nullptr;
  NonlocalDev nl = h->nl;
  const bool prof_contract = h->prof && nonlocal && nl.nseg > 0;
  if (prof_contract) CX_TRY_CUDA(h, cudaEventRecord(h->cev, h->stream));
  if (nonlocal && nl.nseg > 0) {
    nl.node_wchi = sizeof(R) == 4 ? h->d_node_wchi32 : h->d_node_wchi64;
    nl.ent_chi = sizeof(R) == 4 ? h->d_ent_chi32 : h->d_ent_chi64;
    if (sizeof(R) == 4 && h->nltc_contract && h->use_nltc && nl.seg_phase32)
      CX_TRY_CUDA(h, launch_nl_contract_tc(h->g, (const BlockDev<float>*)d_blocks, d_state_tab, nstates, in_sel, nl, h->nltc,
                                           (float2*)cprime, h->d_status, h->stream));
    else
      CX_TRY_CUDA(h, launch_nl_contract<R>(h->g, d_blocks, d_state_tab, nstates, in_sel, nl, cprime, h->stream));
    h->launches++;
    nlp = &nl;
  }
  const bool tma = (sizeof(R) == 4) && maps && h->use_tma;
  if constexpr (sizeof(R) == 4) {
    // autotuner: the first two-array step (idempotent: it does not read its output) over a full
    // state set times every (rows per thread, prefetch depth) configuration twice and keeps the
    // fastest for this handle; every configuration computes the same values
    if (tma && !h->tma_tuned && !use_xprev && nstates >= 64) {
      int rp[24], dp[24];
      const int nc = tma_candidates(h->g, rp, dp, 24);
      cudaEvent_t e0, e1;
      CX_TRY_CUDA(h, cudaEventCreate(&e0));
      CX_TRY_CUDA(h, cudaEventCreate(&e1));
      float best = 1e30f;
      std::string log;
      for (int c = 0; c < nc; ++c) {
        float tmin = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
          CX_TRY_CUDA(h, cudaEventRecord(e0, h->stream));
          CX_TRY_CUDA(h, launch_cheb_step_tma(h->g, h->coef, (const BlockDev<float>*)d_blocks, d_scal, d_state_tab, nstates, in_sel,
                                              use_xprev, *(const TmaMapSet*)maps, h->d_status, h->stream, rp[c], dp[c]));
          CX_TRY_CUDA(h, cudaEventRecord(e1, h->stream));
          CX_TRY_CUDA(h, cudaEventSynchronize(e1));
          float ms = 0;
          CX_TRY_CUDA(h, cudaEventElapsedTime(&ms, e0, e1));
          tmin = std::min(tmin, ms);
        }
        h->launches += 2;
        log += (log.empty() ? "" : " ") + std::to_string(rp[c]) + "/" + std::to_string(dp[c]) + ":" + std::to_string(tmin);
        if (tmin < best) {
          best = tmin;
          h->tma_rpt = rp[c];
          h->tma_depth = dp[c];
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      h->tma_tuned = true;
      h->tma_tuning = log;
    }
  }
  if (h->prof) CX_TRY_CUDA(h, cudaEventRecord(h->ev0, h->stream));
  if constexpr (sizeof(R) == 4) {
    if (tma) {
      // stencil without the projector term, then the projector apply on the touched row chunks
      CX_TRY_CUDA(h, launch_cheb_step_tma(h->g, h->coef, (const BlockDev<float>*)d_blocks, d_scal, d_state_tab, nstates, in_sel,
                                          use_xprev, *(const TmaMapSet*)maps, h->d_status, h->stream, h->tma_rpt, h->tma_depth));
    }
  }
  if (!tma)
    CX_TRY_CUDA(h, launch_cheb_step<R>(h->g, h->coef, d_blocks, d_scal, nblk, d_state_tab, nstates, in_sel, use_xprev, nlp, cprime,
                                       h->stream));
  h->launches++;
  if (h->prof) CX_TRY_CUDA(h, cudaEventRecord(h->ev1, h->stream));
  if (tma && nlp) {
    if (h->nltc_apply && h->use_nltc)
      CX_TRY_CUDA(h, launch_nl_apply_tc(h->g, (const BlockDev<float>*)d_blocks, d_scal, d_state_tab, nstates, in_sel ^ 1, h->chunks32,
                                        h->nltc, (const float2*)cprime, nlp->nseg, h->d_status, h->stream));
    else
      CX_TRY_CUDA(h, launch_nl_apply<R>(h->g, d_blocks, d_scal, d_state_tab, nstates, in_sel ^ 1,
                                        sizeof(R) == 4 ? h->chunks32 : h->chunks64, cprime, nlp->nseg, h->stream));
    h->launches++;
  }
  if (h->prof) {
    CX_TRY_CUDA(h, cudaEventRecord(h->tev1, h->stream));
    CX_TRY_CUDA(h, cudaEventSynchronize(h->tev1));
    float ms = 0, ms2 = 0;
    CX_TRY_CUDA(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    CX_TRY_CUDA(h, cudaEventElapsedTime(&ms2, h->ev1, h->tev1));
    if (prof_contract) {
      float ms3 = 0;
      CX_TRY_CUDA(h, cudaEventElapsedTime(&ms3, h->cev, h->ev0));
      h->prof_contract_ms += ms3;
    }
    h->prof_ms += ms;
    h->prof_apply_ms += ms2;
    h->prof_launches++;
    h->prof_bytes += bytes;
  }
  return CX_OK;
}

// Filter degree m on all blocks of the set; psi in buffer sel0, result buffer returned in *sel_out.
template <typename R>
cx_status filter_blocks(cx_handle h, const BlockDev<R>* d_blocks, int nblk, const int2* d_state_tab, int nstates,
                        size_t total_elems, int sel0, int m, const std::vector<double>& a, const std::vector<double>& b,
                        const std::vector<double>& a0, cplx<R>* cprime, int* sel_out, const void* maps) {
  if (m < 1) { h->err = "filter degree must be >= 1"; return CX_ERR_ARG; }
  std::vector<StepScalars> sc((size_t)m * nblk);
  for (int i = 0; i < nblk; ++i) cheb_scalars(m, a[i], b[i], a0[i], sc, nblk, i);
  if (h->scal_cap < m * nblk) {
    cudaFree(h->d_scal);
    h->d_scal = nullptr;
    h->scal_cap = 0;
    cx_status s = dalloc(h, &h->d_scal, (size_t)m * nblk);
    if (s != CX_OK) return s;
    h->scal_cap = m * nblk;
  }
  CX_TRY_CUDA(h, cudaMemcpyAsync(h->d_scal, sc.data(), sc.size() * sizeof(StepScalars), cudaMemcpyHostToDevice, h->stream));
  const double sz = (double)total_elems * sizeof(cplx<R>);
  for (int d = 1; d <= m; ++d) {
    const int in_sel = sel0 ^ ((d - 1) & 1);
    cx_status s = fused_step<R>(h, d_blocks, h->d_scal + (size_t)(d - 1) * nblk, nblk, d_state_tab, nstates, in_sel, d >= 2,
                                cprime, true, (d >= 2 ? 3.0 : 2.0) * sz, maps);
    if (s != CX_OK) return s;
  }
  *sel_out = sel0 ^ (m & 1);
  return CX_OK;
}

template cx_status filter_blocks<float>(cx_handle, const BlockDev<float>*, int, const int2*, int, size_t, int, int,
                                        const std::vector<double>&, const std::vector<double>&, const std::vector<double>&,
                                        cplx<float>*, int*, const void*);
template cx_status filter_blocks<double>(cx_handle, const BlockDev<double>*, int, const int2*, int, size_t, int, int,
                                         const std::vector<double>&, const std::vector<double>&, const std::vector<double>&,
                                         cplx<double>*, int*, const void*);
template cx_status make_block_devs<float>(cx_handle, const std::vector<cplx<float>*>&, const std::vector<cplx<float>*>&,
                                          const std::vector<int>&, std::vector<BlockDev<float>>&);
template cx_status make_block_devs<double>(cx_handle, const std::vector<cplx<double>*>&, const std::vector<cplx<double>*>&,
                                           const std::vector<int>&, std::vector<BlockDev<double>>&);
template cx_status fused_step<float>(cx_handle, const BlockDev<float>*, const StepScalars*, int, const int2*, int, int, bool,
                                     cplx<float>*, bool, double, const void*);
template cx_status fused_step<double>(cx_handle, const BlockDev<double>*, const StepScalars*, int, const int2*, int, int, bool,
                                      cplx<double>*, bool, double, const void*);

cx_status build_maps(cx_handle h, const std::vector<const void*>& p0, const std::vector<const void*>& p1, const std::vector<int>& Ns,
                     void** d_maps, TmaMapSet* set) {
  *d_maps = nullptr;
  const size_t nb = p0.size();
  // [nb][2] staged-row maps, then [nb][2] theta-halo maps, then [nb][2] output-tile maps
  std::vector<CUtensorMap_st> maps(6 * nb);
  for (size_t b = 0; b < nb; ++b) {
    cx_status s = make_buffer_maps(h, p0[b], Ns[b], &maps[2 * b], &maps[2 * nb + 2 * b], &maps[4 * nb + 2 * b]);
    if (s != CX_OK) return s;
    if ((s = make_buffer_maps(h, p1[b], Ns[b], &maps[2 * b + 1], &maps[2 * nb + 2 * b + 1], &maps[4 * nb + 2 * b + 1])) != CX_OK)
      return s;
  }
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, maps.size() * sizeof(CUtensorMap_st));
  if (e != cudaSuccess) { h->err = std::string("tensor maps: ") + cudaGetErrorString(e); return CX_ERR_NOMEM; }
  e = cudaMemcpy(d, maps.data(), maps.size() * sizeof(CUtensorMap_st), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(d); h->err = std::string("tensor maps: ") + cudaGetErrorString(e); return CX_ERR_CUDA; }
  *d_maps = d;
  set->xmaps = d;
  set->hmaps = (const CUtensorMap_st*)d + 2 * nb;
  set->omaps = (const CUtensorMap_st*)d + 4 * nb;
  set->vmaps = h->d_fmaps;
  return CX_OK;
}

cx_status check_pipeline_status(cx_handle h) {
  if (!h->d_status) return CX_OK;
  int st = 0;
  CX_TRY_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  if (st != 0) {
    CX_TRY_CUDA(h, cudaMemset(h->d_status, 0, sizeof(int)));
    h->err = "stencil pipeline: a bulk-copy wait exceeded its iteration limit (results of this call are invalid)";
    return CX_ERR_CUDA;
  }
  return CX_OK;
}

// A one-block scratch view (used by the host-buffer entry points): temporary buffers of ncol columns.
template <typename R>
struct ScratchView {
  cplx<R>* b0 = nullptr;
  cplx<R>* b1 = nullptr;
  cplx<R>* cprime = nullptr;
  BlockDev<R>* d_blk = nullptr;
  int2* d_tab = nullptr;
  StepScalars* d_scal = nullptr;
  double2* d_ph = nullptr;
  void* d_maps = nullptr;
  TmaMapSet set{};
  ~ScratchView() {
    cudaFree(b0); cudaFree(b1); cudaFree(cprime); cudaFree(d_blk); cudaFree(d_tab); cudaFree(d_scal); cudaFree(d_ph);
    cudaFree(d_maps);
  }
};

template <typename R>
cx_status make_scratch(cx_handle h, int blk, int ncol, ScratchView<R>& v) {
  const size_t N = h->g.N;
  cx_status s;
  if ((s = dalloc(h, &v.b0, N * ncol)) != CX_OK) return s;
  if ((s = dalloc(h, &v.b1, N * ncol)) != CX_OK) return s;
  const int nseg = std::max(1, h->nl.nseg);
  if ((s = dalloc(h, &v.cprime, (size_t)ncol * nseg * kAngMax)) != CX_OK) return s;
  if ((s = dalloc(h, &v.d_blk, 1)) != CX_OK) return s;
  if ((s = dalloc(h, &v.d_tab, ncol)) != CX_OK) return s;
  if ((s = dalloc(h, &v.d_ph, nseg)) != CX_OK) return s;
  std::vector<BlockDev<R>> bd;
  std::vector<cplx<R>*> p0{v.b0}, p1{v.b1};
  make_block_devs<R>(h, p0, p1, std::vector<int>{blk}, bd);
  bd[0].Ns = ncol;
  CX_TRY_CUDA(h, cudaMemcpy(v.d_blk, bd.data(), sizeof(BlockDev<R>), cudaMemcpyHostToDevice));
  std::vector<int2> tab(ncol);
  for (int i = 0; i < ncol; ++i) tab[i] = make_int2(0, i);
  CX_TRY_CUDA(h, cudaMemcpy(v.d_tab, tab.data(), sizeof(int2) * ncol, cudaMemcpyHostToDevice));
  std::vector<double2> ph = segment_phases(h, h->blocks[blk]);
  if (!ph.empty()) CX_TRY_CUDA(h, cudaMemcpy(v.d_ph, ph.data(), sizeof(double2) * ph.size(), cudaMemcpyHostToDevice));
  if (sizeof(R) == 4 && h->tma_ok) {
    if ((s = build_maps(h, {v.b0}, {v.b1}, {ncol}, &v.d_maps, &v.set)) != CX_OK) return s;
  }
  return CX_OK;
}

template <typename R>
static cx_status hpsi_T(cx_handle h, int blk, int ncol, const double* X, double* Y) {
  ScratchView<R> v;
  cx_status s = make_scratch<R>(h, blk, ncol, v);
  if (s != CX_OK) return s;
  const size_t n = (size_t)h->g.N * ncol;
  if ((s = cx_host_to_dev(h, X, v.b0, n, sizeof(R) == 8 ? CX_PREC_FP64 : CX_PREC_MIXED)) != CX_OK) return s;
  StepScalars one{1.0, 0.0, 0.0, 0.0};
  if ((s = dalloc(h, &v.d_scal, 1)) != CX_OK) return s;
  CX_TRY_CUDA(h, cudaMemcpy(v.d_scal, &one, sizeof(one), cudaMemcpyHostToDevice));
  const double2* saved = h->nl.seg_phase;
  const float2* saved32 = h->nl.seg_phase32;
  h->nl.seg_phase = v.d_ph;
  h->nl.seg_phase32 = nullptr;
  s = fused_step<R>(h, v.d_blk, v.d_scal, 1, v.d_tab, ncol, 0, false, v.cprime, true, 2.0 * n * sizeof(cplx<R>), v.d_maps ? &v.set : nullptr);
  h->nl.seg_phase = saved;
  h->nl.seg_phase32 = saved32;
  if (s != CX_OK) return s;
  if ((s = check_pipeline_status(h)) != CX_OK) return s;
  return cx_dev_to_host(h, v.b1, Y, n, sizeof(R) == 8 ? CX_PREC_FP64 : CX_PREC_MIXED);
}

template <typename R>
static cx_status filter_T(cx_handle h, int blk, int ncol, const double* X, double* Y, int m, double a, double b, double a0) {
  ScratchView<R> v;
  cx_status s = make_scratch<R>(h, blk, ncol, v);
  if (s != CX_OK) return s;
  const size_t n = (size_t)h->g.N * ncol;
  const int pr = sizeof(R) == 8 ? CX_PREC_FP64 : CX_PREC_MIXED;
  if ((s = cx_host_to_dev(h, X, v.b0, n, pr)) != CX_OK) return s;
  const double2* saved = h->nl.seg_phase;
  const float2* saved32 = h->nl.seg_phase32;
  h->nl.seg_phase = v.d_ph;
  h->nl.seg_phase32 = nullptr;
  StepScalars* saved_scal = h->d_scal;
  int saved_cap = h->scal_cap;
  h->d_scal = nullptr;
  h->scal_cap = 0;
  int sel = 0;
  s = filter_blocks<R>(h, v.d_blk, 1, v.d_tab, ncol, n, 0, m, std::vector<double>{a}, std::vector<double>{b},
                       std::vector<double>{a0}, v.cprime, &sel, v.d_maps ? &v.set : nullptr);
  if (s == CX_OK) s = check_pipeline_status(h);
  v.d_scal = h->d_scal;            // freed with the view
  h->d_scal = saved_scal;
  h->scal_cap = saved_cap;
  h->nl.seg_phase = saved;
  h->nl.seg_phase32 = saved32;
  if (s != CX_OK) return s;
  return cx_dev_to_host(h, sel ? v.b1 : v.b0, Y, n, pr);
}

}  // namespace cx

using namespace cx;

extern "C" {

const char* cx_version(void) { return "cyclix_gpu 0.1 (sm_103a)"; }

cx_status cx_set_device(int32_t device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    g_create_err = "cx_set_device: no such device";
    return CX_ERR_ARG;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    g_create_err = "cx_set_device: cudaSetDevice failed";
    return CX_ERR_CUDA;
  }
  return CX_OK;
}

const char* cx_last_error(cx_handle h) { return h ? h->err.c_str() : g_create_err.c_str(); }

cx_status cx_create(const cx_grid* grid, int32_t n_atm, const cx_atom* atoms, int32_t nspin, cx_handle* out) {
  if (!out) { g_create_err = "cx_create: out is NULL"; return CX_ERR_ARG; }
  *out = nullptr;
  if (!grid || !grid->w1 || !grid->w2 || !grid->W) { g_create_err = "cx_create: grid, w1, w2, W required"; return CX_ERR_ARG; }
  const cx_grid& G = *grid;
  if (G.FDn < 1 || G.FDn > kMaxFDn) { g_create_err = "cx_create: FDn must be in 1..8"; return CX_ERR_ARG; }
  if (G.cell_typ < 3 || G.cell_typ > 5) { g_create_err = "cx_create: cell_typ must be 3 (cyclic) or 4/5 (helical)"; return CX_ERR_ARG; }
  if (G.BCx != 1) { g_create_err = "cx_create: the radial direction must be Dirichlet (BCx = 1)"; return CX_ERR_ARG; }
  if (G.Nx < 1 || G.Ny <= G.FDn || G.Nz <= G.FDn) {
    g_create_err = "cx_create: need Nx >= 1 and Ny, Nz > FDn (one Bloch wrap per stencil)";
    return CX_ERR_ARG;
  }
  if ((G.cell_typ == 4 || G.cell_typ == 5) && G.twist == 0) { g_create_err = "cx_create: helical cell needs twist != 0"; return CX_ERR_ARG; }
  if (nspin < 1 || nspin > 2) { g_create_err = "cx_create: nspin must be 1 or 2"; return CX_ERR_ARG; }
  if (n_atm < 0 || (n_atm > 0 && !atoms)) { g_create_err = "cx_create: atoms required"; return CX_ERR_ARG; }
  const long long Nll = (long long)G.Nx * G.Ny * G.Nz;
  if (Nll >= (1LL << 31)) { g_create_err = "cx_create: grid too large (N must fit int32)"; return CX_ERR_ARG; }
  // projector columns per atom: the kernels hold kAngMax (l <= 1, one projector per l); a psp8
  // atom with two projectors per l has 8 and is refused here, before any CUDA work
  for (int J = 0; J < n_atm; ++J) {
    const cx_atom& A = atoms[J];
    if (A.angnum < 0 || A.angnum > kAngMax || A.n_image_rc < 0 || (A.n_image_rc > 0 && !A.rcImage) || (A.angnum > 0 && !A.gamma_Jl)) {
      g_create_err = "cx_create: atom " + std::to_string(J) + ": angnum must be 0.." + std::to_string(kAngMax) +
                     " (got " + std::to_string(A.angnum) + ") and rcImage/gamma_Jl given";
      return CX_ERR_ARG;
    }
  }

  cx_handle h = new cx_handle_s();
  h->grid = G;
  h->nspin = nspin;
  const int N = (int)Nll;
  h->g.Nx = G.Nx; h->g.Ny = G.Ny; h->g.Nz = G.Nz; h->g.N = N;
  h->g.FDn = G.FDn; h->g.helical = (G.cell_typ != 3); h->g.BCy = G.BCy; h->g.BCz = G.BCz;
  h->g.xin = G.xin; h->g.dx = G.dx; h->g.twist = G.twist;
  // 1-D stencil coefficients (Cychel/lapIndicesValues_1d_cychel.m:30-46,165-173,191-201,229-239)
  for (int q = 0; q <= G.FDn; ++q) {
    h->coef.cr2[q] = G.w2[q] / (G.dx * G.dx);
    h->coef.cr1[q] = q == 0 ? 0.0 : G.w1[q] / G.dx;
    h->coef.ct2[q] = G.w2[q] / (G.dy * G.dy);
    h->coef.ct1[q] = q == 0 ? 0.0 : -2.0 * G.twist * G.w1[q] / G.dy;
    h->coef.cz2[q] = G.w2[q] / (G.dz * G.dz);
    h->coef.cz1[q] = q == 0 ? 0.0 : G.w1[q] / G.dz;
    h->w1[q] = G.w1[q];
  }
  h->W.assign(G.W, G.W + N);
  cudaError_t e;
  if ((e = cudaGetDevice(&h->dev)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    g_create_err = std::string("cx_create: CUDA unavailable: ") + cudaGetErrorString(e);
    delete h;
    return CX_ERR_CUDA;
  }
  cudaEventCreate(&h->ev0); cudaEventCreate(&h->ev1); cudaEventCreate(&h->tev0); cudaEventCreate(&h->tev1);
  cudaEventCreate(&h->cev);
  for (auto& e : h->eig_ev) cudaEventCreate(&e);
  if (cublasCreate(&h->cublas) != CUBLAS_STATUS_SUCCESS || cublasSetStream(h->cublas, h->stream) != CUBLAS_STATUS_SUCCESS) {
    g_create_err = "cx_create: cublasCreate failed";
    cx_destroy(h);
    return CX_ERR_LIB;
  }
  if (cusolverDnCreate(&h->cusolver) != CUSOLVER_STATUS_SUCCESS || cusolverDnSetStream(h->cusolver, h->stream) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnCreateParams(&h->cusolver_params) != CUSOLVER_STATUS_SUCCESS) {
    g_create_err = "cx_create: cusolverDnCreate failed";
    cx_destroy(h);
    return CX_ERR_LIB;
  }
  cx_status s;
  if ((s = upload(h, &h->d_W, h->W)) != CX_OK) { g_create_err = h->err; cx_destroy(h); return s; }
  {
    const std::vector<float> w32(h->W.begin(), h->W.end());
    if ((s = upload(h, &h->d_W32, w32)) != CX_OK) { g_create_err = h->err; cx_destroy(h); return s; }
  }
  if ((s = dalloc(h, &h->d_veff, (size_t)N * nspin)) != CX_OK) { g_create_err = h->err; cx_destroy(h); return s; }
  if ((s = dalloc(h, &h->d_status, 1)) != CX_OK) { g_create_err = h->err; cx_destroy(h); return s; }
  CX_TRY_CUDA(h, cudaMemset(h->d_status, 0, sizeof(int)));
  CX_TRY_CUDA(h, cudaMemset(h->d_veff, 0, sizeof(double) * (size_t)N * nspin));

  // ---- nonlocal tables
  std::vector<int32_t> atom_node_ptr(1, 0), node_pos, node_seg, atom_seg_ptr(1, 0), angn;
  std::vector<double> node_wchi, gam;
  std::vector<int32_t> ent_count(N, 0);
  for (int J = 0; J < n_atm; ++J) {
    const cx_atom& A = atoms[J];
    if (A.angnum < 0 || A.angnum > kAngMax || A.n_image_rc < 0 || (A.n_image_rc > 0 && !A.rcImage) || (A.angnum > 0 && !A.gamma_Jl)) {
      g_create_err = "cx_create: atom " + std::to_string(J) + ": angnum must be 0..4 and rcImage/gamma_Jl given";
      cx_destroy(h);
      return CX_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d) h->atom_pos.push_back(A.position[d]);
    for (int q = 0; q < kAngMax; ++q) gam.push_back(q < A.angnum ? A.gamma_Jl[q] : 0.0);
    angn.push_back(A.angnum);
    for (int im = 0; im < A.n_image_rc; ++im) {
      const cx_rc_image& I = A.rcImage[im];
      const int seg = (int)h->seg_atom.size();
      h->seg_atom.push_back(J);
      for (int d = 0; d < 3; ++d) h->seg_coord.push_back(I.coordinates[d]);
      if (I.rc_n_nodes < 0 || (I.rc_n_nodes > 0 && (!I.rc_pos || !I.Chi_mat))) {
        g_create_err = "cx_create: image without rc_pos / Chi_mat";
        cx_destroy(h);
        return CX_ERR_ARG;
      }
      for (int n = 0; n < I.rc_n_nodes; ++n) {
        const int64_t pos = I.rc_pos[n] - 1;
        if (pos < 0 || pos >= N) {
          g_create_err = "cx_create: rc_pos out of range (atom " + std::to_string(J) + ")";
          cx_destroy(h);
          return CX_ERR_ARG;
        }
        node_pos.push_back((int32_t)pos);
        node_seg.push_back(seg);
        for (int q = 0; q < kAngMax; ++q)
          node_wchi.push_back(q < A.angnum ? h->W[pos] * I.Chi_mat[(size_t)q * I.rc_n_nodes + n] : 0.0);
        ent_count[pos]++;
      }
    }
    atom_node_ptr.push_back((int32_t)node_pos.size());
    atom_seg_ptr.push_back((int32_t)h->seg_atom.size());
  }
  // per-point CSR of (segment, Chi) entries for the fused apply
  std::vector<int32_t> row_ptr(N + 1, 0);
  for (int p = 0; p < N; ++p) row_ptr[p + 1] = row_ptr[p] + ent_count[p];
  const size_t nent = row_ptr[N];
  std::vector<int32_t> ent_seg(nent), fill(row_ptr.begin(), row_ptr.end() - 1);
  std::vector<double> ent_chi(nent * kAngMax, 0.0);
  {
    size_t n = 0;
    for (int J = 0; J < n_atm; ++J) {
      const cx_atom& A = atoms[J];
      for (int im = 0; im < A.n_image_rc; ++im) {
        const cx_rc_image& I = A.rcImage[im];
        for (int k = 0; k < I.rc_n_nodes; ++k, ++n) {
          const int p = node_pos[n];
          const int slot = fill[p]++;
          ent_seg[slot] = node_seg[n];
          for (int q = 0; q < A.angnum; ++q) ent_chi[(size_t)slot * kAngMax + q] = I.Chi_mat[(size_t)q * I.rc_n_nodes + k];
        }
      }
    }
  }
  h->nl.n_atm = n_atm;
  h->nl.nseg = (int)h->seg_atom.size();
  h->nl.nnode = (int)node_pos.size();
  std::vector<float> node_wchi32(node_wchi.begin(), node_wchi.end()), ent_chi32(ent_chi.begin(), ent_chi.end());
  int32_t *d_anp, *d_np, *d_ns, *d_asp, *d_an, *d_rp, *d_es;
  double *d_g, *d_w64, *d_c64;
  float *d_w32, *d_c32;
  if ((s = upload(h, &d_anp, atom_node_ptr)) || (s = upload(h, &d_np, node_pos)) || (s = upload(h, &d_ns, node_seg)) ||
      (s = upload(h, &d_asp, atom_seg_ptr)) || (s = upload(h, &d_an, angn)) || (s = upload(h, &d_rp, row_ptr)) ||
      (s = upload(h, &d_es, ent_seg)) || (s = upload(h, &d_g, gam)) || (s = upload(h, &d_w64, node_wchi)) ||
      (s = upload(h, &d_c64, ent_chi)) || (s = upload(h, &d_w32, node_wchi32)) || (s = upload(h, &d_c32, ent_chi32))) {
    g_create_err = h->err;
    cx_destroy(h);
    return s;
  }
  h->nl.atom_node_ptr = d_anp; h->nl.node_pos = d_np; h->nl.node_seg = d_ns; h->nl.atom_seg_ptr = d_asp;
  h->nl.angnum = d_an; h->nl.row_ptr = d_rp; h->nl.ent_seg = d_es; h->nl.gamma = d_g;
  h->d_node_wchi64 = d_w64; h->d_ent_chi64 = d_c64; h->d_node_wchi32 = d_w32; h->d_ent_chi32 = d_c32;
  {
    // tensor-core contraction operands (W Chi per atom, hi / lo tf32 in the MMA layout)
    std::vector<int64_t> iptr;
    std::vector<float> img;
    if (n_atm > 0 && nl_tc_contract_images(atom_node_ptr, node_seg, atom_seg_ptr, node_wchi, iptr, img) && !img.empty()) {
      int64_t* d_ip;
      float* d_im;
      if ((s = upload(h, &d_ip, iptr)) || (s = upload(h, &d_im, img))) { g_create_err = h->err; cx_destroy(h); return s; }
      h->nltc.ct_ptr = d_ip;
      h->nltc.ct_img = d_im;
      h->nltc_contract = true;
    }
  }
  // TMA path: per-point entry start / count, float Veff and the field maps
  h->tma_ok = tma_eligible(h->g, sizeof(float2));
  if (h->tma_ok) {
    // 32-point row chunks that projector balls touch, each with its segments and dense Chi
    std::vector<int32_t> cp0, cseg_ptr(1, 0), csegs;
    std::vector<int64_t> cchi_ptr;
    std::vector<double> cchi;
    int kmax = 0;
    for (int row = 0; row < N / G.Nx; ++row)
      for (int r0 = 0; r0 < G.Nx; r0 += 32) {
        const int p0 = row * G.Nx + r0, p1 = std::min(p0 + 32, (row + 1) * G.Nx);
        if (row_ptr[p1] == row_ptr[p0]) continue;
        std::vector<int32_t> sg;
        for (int e = row_ptr[p0]; e < row_ptr[p1]; ++e) sg.push_back(ent_seg[e]);
        std::sort(sg.begin(), sg.end());
        sg.erase(std::unique(sg.begin(), sg.end()), sg.end());
        const int K = (int)sg.size() * kAngMax;
        kmax = std::max(kmax, K);
        cp0.push_back(p0);
        csegs.insert(csegs.end(), sg.begin(), sg.end());
        cseg_ptr.push_back((int32_t)csegs.size());
        cchi_ptr.push_back((int64_t)cchi.size());
        const size_t base = cchi.size();
        cchi.resize(base + (size_t)K * 32, 0.0);
        for (int p = p0; p < p1; ++p)
          for (int e = row_ptr[p]; e < row_ptr[p + 1]; ++e) {
            const int ls = (int)(std::lower_bound(sg.begin(), sg.end(), ent_seg[e]) - sg.begin());
            for (int q = 0; q < kAngMax; ++q) cchi[base + (size_t)(ls * kAngMax + q) * 32 + (p - p0)] = ent_chi[(size_t)e * kAngMax + q];
          }
      }
    std::vector<float> cchi32(cchi.begin(), cchi.end());
    int32_t *d_cp0, *d_csp, *d_csg;
    int64_t* d_ccp;
    double* d_cc64;
    float* d_cc32;
    if ((s = upload(h, &d_cp0, cp0)) || (s = upload(h, &d_csp, cseg_ptr)) || (s = upload(h, &d_csg, csegs)) ||
        (s = upload(h, &d_ccp, cchi_ptr)) || (s = upload(h, &d_cc64, cchi)) || (s = upload(h, &d_cc32, cchi32)) ||
        (s = dalloc(h, &h->d_veff32, (size_t)N * nspin))) {
      g_create_err = h->err;
      cx_destroy(h);
      return s;
    }
    h->chunks32 = ChunkTables{(int32_t)cp0.size(), kmax, d_cp0, d_csp, d_csg, d_ccp, d_cc32};
    if (!cp0.empty()) {
      // tensor-core apply operands (Chi per chunk, hi / lo tf32 in the MMA layout)
      std::vector<int64_t> iptr;
      std::vector<float> img;
      nl_tc_apply_images(cseg_ptr, cchi_ptr, cchi, iptr, img);
      int64_t* d_ip;
      float* d_im;
      if ((s = upload(h, &d_ip, iptr)) || (s = upload(h, &d_im, img))) { g_create_err = h->err; cx_destroy(h); return s; }
      h->nltc.ap_ptr = d_ip;
      h->nltc.ap_img = d_im;
      h->nltc_apply = true;
    }
    h->chunks64 = ChunkTables{(int32_t)cp0.size(), kmax, d_cp0, d_csp, d_csg, d_ccp, d_cc64};
    CX_TRY_CUDA(h, cudaMemset(h->d_veff32, 0, sizeof(float) * (size_t)N * nspin));
    std::vector<CUtensorMap_st> fm(nspin);
    for (int sp = 0; sp < nspin; ++sp)
      if ((s = make_field_map(h, h->d_veff32 + (size_t)sp * N, false, &fm[sp])) != CX_OK) { g_create_err = h->err; cx_destroy(h); return s; }
    if (cudaMalloc(&h->d_fmaps, fm.size() * sizeof(CUtensorMap_st)) != cudaSuccess ||
        cudaMemcpy(h->d_fmaps, fm.data(), fm.size() * sizeof(CUtensorMap_st), cudaMemcpyHostToDevice) != cudaSuccess) {
      g_create_err = "cx_create: field tensor maps";
      cx_destroy(h);
      return CX_ERR_NOMEM;
    }
  }
  *out = h;
  return CX_OK;
}

cx_status cx_destroy(cx_handle h) {
  if (!h) return CX_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_blocks(h);
  for (void* p : h->nl_allocs) cudaFree(p);
  cudaFree(h->d_veff);
  cudaFree(h->d_veff32);
  cudaFree(h->d_fmaps);
  cudaFree(h->d_status);
  cudaFree(h->d_scal);
  cudaFree(h->d_ws);
  cudaFreeHost(h->h_ws);
  cx_free_extra(h);
  if (h->cusolver_params) cusolverDnDestroyParams(h->cusolver_params);
  if (h->cusolver) cusolverDnDestroy(h->cusolver);
  if (h->cublas) cublasDestroy(h->cublas);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->tev0) cudaEventDestroy(h->tev0);
  if (h->tev1) cudaEventDestroy(h->tev1);
  if (h->cev) cudaEventDestroy(h->cev);
  for (auto& e : h->eig_ev)
    if (e) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return CX_OK;
}

__global__ void k_veff32(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

cx_status cx_set_veff(cx_handle h, const double* Veff) {
  if (!h || !Veff) return CX_ERR_ARG;
  CX_TRY_CUDA(h, cudaMemcpyAsync(h->d_veff, Veff, sizeof(double) * (size_t)h->g.N * h->nspin, cudaMemcpyHostToDevice, h->stream));
  if (h->d_veff32) {
    const size_t n = (size_t)h->g.N * h->nspin;
    k_veff32<<<(unsigned)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, h->stream>>>(h->d_veff, h->d_veff32, n);
    h->launches++;
    CX_TRY_CUDA(h, cudaGetLastError());
  }
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  return CX_OK;
}

cx_status cx_set_blocks(cx_handle h, int32_t nblk, const cx_block* blocks, int32_t prec) {
  if (!h) return CX_ERR_ARG;
  if (nblk < 1 || !blocks) { h->err = "cx_set_blocks: need nblk >= 1 blocks"; return CX_ERR_ARG; }
  if (prec != CX_PREC_FP64 && prec != CX_PREC_MIXED) { h->err = "cx_set_blocks: prec must be CX_PREC_FP64 or CX_PREC_MIXED"; return CX_ERR_ARG; }
  int total = 0;
  for (int b = 0; b < nblk; ++b) {
    if (blocks[b].Ns < 1 || blocks[b].spin < 0 || blocks[b].spin >= h->nspin) {
      h->err = "cx_set_blocks: block " + std::to_string(b) + " needs Ns >= 1 and 0 <= spin < nspin";
      return CX_ERR_ARG;
    }
    total += blocks[b].Ns;
  }
  if (total > 65535) { h->err = "cx_set_blocks: at most 65535 states in total"; return CX_ERR_ARG; }
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  free_blocks(h);
  h->prec = prec;
  h->nblk = nblk;
  h->blocks.assign(blocks, blocks + nblk);
  const size_t N = h->g.N;
  const size_t cs = prec == CX_PREC_FP64 ? sizeof(double2) : sizeof(float2);
  std::vector<int2> tab;
  for (int b = 0; b < nblk; ++b) {
    h->state0.push_back(h->nstates);
    for (int i = 0; i < blocks[b].Ns; ++i) tab.push_back(make_int2(b, i));
    h->nstates += blocks[b].Ns;
    for (int k = 0; k < 2; ++k) {
      void* p = nullptr;
      cudaError_t e = cudaMalloc(&p, N * blocks[b].Ns * cs);
      if (e != cudaSuccess) { h->err = std::string("cx_set_blocks: psi buffers: ") + cudaGetErrorString(e); free_blocks(h); return CX_ERR_NOMEM; }
      h->bufs.push_back(p);
    }
    void* u = nullptr;
    if (cudaMalloc(&u, N * sizeof(double2)) != cudaSuccess) { h->err = "cx_set_blocks: bound vectors"; free_blocks(h); return CX_ERR_NOMEM; }
    cudaMemset(u, 0, N * sizeof(double2));
    h->ubgv.push_back(u);
  }
  h->psi_sel.assign(1, 0);
  cx_status s;
  if ((s = dalloc(h, &h->d_state_tab, tab.size())) != CX_OK) { free_blocks(h); return s; }
  CX_TRY_CUDA(h, cudaMemcpy(h->d_state_tab, tab.data(), sizeof(int2) * tab.size(), cudaMemcpyHostToDevice));
  const int nseg = std::max(1, h->nl.nseg);
  {
    void* p = nullptr;
    if (cudaMalloc(&p, (size_t)h->nstates * nseg * kAngMax * cs) != cudaSuccess) { h->err = "cx_set_blocks: projector coefficients"; free_blocks(h); return CX_ERR_NOMEM; }
    h->d_cprime = p;
  }
  std::vector<double2> ph;
  for (int b = 0; b < nblk; ++b) {
    std::vector<double2> p = segment_phases(h, blocks[b]);
    if (p.empty()) p.push_back(make_double2(1, 0));
    ph.insert(ph.end(), p.begin(), p.end());
  }
  if ((s = dalloc(h, &h->d_seg_phase, ph.size())) != CX_OK) { free_blocks(h); return s; }
  CX_TRY_CUDA(h, cudaMemcpy(h->d_seg_phase, ph.data(), sizeof(double2) * ph.size(), cudaMemcpyHostToDevice));
  h->nl.seg_phase = h->d_seg_phase;
  {
    std::vector<float2> ph32(ph.size());
    for (size_t i = 0; i < ph.size(); ++i) ph32[i] = make_float2((float)ph[i].x, (float)ph[i].y);
    if (cudaMalloc(&h->d_seg_phase32, sizeof(float2) * std::max<size_t>(1, ph32.size())) != cudaSuccess) {
      h->err = "cx_set_blocks: device memory for the segment phases";
      free_blocks(h);
      return CX_ERR_NOMEM;
    }
    CX_TRY_CUDA(h, cudaMemcpy(h->d_seg_phase32, ph32.data(), sizeof(float2) * ph32.size(), cudaMemcpyHostToDevice));
    h->nl.seg_phase32 = h->d_seg_phase32;
  }
  std::vector<int> ids(nblk);
  for (int b = 0; b < nblk; ++b) ids[b] = b;
  if (prec == CX_PREC_FP64) {
    std::vector<cplx<double>*> p0, p1;
    for (int b = 0; b < nblk; ++b) { p0.push_back((cplx<double>*)h->bufs[2 * b]); p1.push_back((cplx<double>*)h->bufs[2 * b + 1]); }
    std::vector<BlockDev<double>> bd;
    make_block_devs<double>(h, p0, p1, ids, bd);
    BlockDev<double>* d = nullptr;
    if ((s = dalloc(h, &d, bd.size())) != CX_OK) { free_blocks(h); return s; }
    CX_TRY_CUDA(h, cudaMemcpy(d, bd.data(), sizeof(bd[0]) * bd.size(), cudaMemcpyHostToDevice));
    h->d_blocks = d;
  } else {
    std::vector<cplx<float>*> p0, p1;
    for (int b = 0; b < nblk; ++b) { p0.push_back((cplx<float>*)h->bufs[2 * b]); p1.push_back((cplx<float>*)h->bufs[2 * b + 1]); }
    std::vector<BlockDev<float>> bd;
    make_block_devs<float>(h, p0, p1, ids, bd);
    BlockDev<float>* d = nullptr;
    if ((s = dalloc(h, &d, bd.size())) != CX_OK) { free_blocks(h); return s; }
    CX_TRY_CUDA(h, cudaMemcpy(d, bd.data(), sizeof(bd[0]) * bd.size(), cudaMemcpyHostToDevice));
    h->d_blocks = d;
    if (h->tma_ok) {
      std::vector<const void*> q0(p0.begin(), p0.end()), q1(p1.begin(), p1.end());
      std::vector<int> ns;
      for (int b = 0; b < nblk; ++b) ns.push_back(blocks[b].Ns);
      if ((s = build_maps(h, q0, q1, ns, &h->d_maps, &h->tma_main)) != CX_OK) { free_blocks(h); return s; }
    }
  }
  return CX_OK;
}

cx_status cx_set_psi(cx_handle h, int32_t blk, const double* psi) {
  if (!h || !psi) return CX_ERR_ARG;
  if (blk < 0 || blk >= h->nblk) { h->err = "cx_set_psi: block index out of range"; return CX_ERR_ARG; }
  const size_t n = (size_t)h->g.N * h->blocks[blk].Ns;
  void* dst = h->bufs[2 * blk + h->psi_sel[0]];
  return cx_host_to_dev(h, psi, dst, n, h->prec);
}

cx_status cx_get_psi(cx_handle h, int32_t blk, double* psi) {
  if (!h || !psi) return CX_ERR_ARG;
  if (blk < 0 || blk >= h->nblk) { h->err = "cx_get_psi: block index out of range"; return CX_ERR_ARG; }
  const size_t n = (size_t)h->g.N * h->blocks[blk].Ns;
  const void* src = h->bufs[2 * blk + h->psi_sel[0]];
  return cx_dev_to_host(h, src, psi, n, h->prec);
}

cx_status cx_hpsi(cx_handle h, int32_t blk, int32_t ncol, const double* X, double* Y, int32_t prec) {
  if (!h || !X || !Y) return CX_ERR_ARG;
  if (blk < 0 || blk >= h->nblk) { h->err = "cx_hpsi: block index out of range (call cx_set_blocks first)"; return CX_ERR_STATE; }
  if (ncol < 1 || ncol > 65535) { h->err = "cx_hpsi: ncol must be in 1..65535"; return CX_ERR_ARG; }
  if (prec == CX_PREC_FP64) return hpsi_T<double>(h, blk, ncol, X, Y);
  if (prec == CX_PREC_MIXED) return hpsi_T<float>(h, blk, ncol, X, Y);
  h->err = "cx_hpsi: bad prec";
  return CX_ERR_ARG;
}

cx_status cx_chebyshev_filter(cx_handle h, int32_t blk, int32_t ncol, const double* X, double* Y, int32_t m, double a, double b,
                              double a0, int32_t prec) {
  if (!h || !X || !Y) return CX_ERR_ARG;
  if (blk < 0 || blk >= h->nblk) { h->err = "cx_chebyshev_filter: block index out of range (call cx_set_blocks first)"; return CX_ERR_STATE; }
  if (ncol < 1 || ncol > 65535 || m < 1) { h->err = "cx_chebyshev_filter: need 1 <= ncol <= 65535 and m >= 1"; return CX_ERR_ARG; }
  if (!(b > a) || !(a > a0)) { h->err = "cx_chebyshev_filter: need a0 < a < b (lower bound < cutoff < upper bound)"; return CX_ERR_ARG; }
  if (prec == CX_PREC_FP64) return filter_T<double>(h, blk, ncol, X, Y, m, a, b, a0);
  if (prec == CX_PREC_MIXED) return filter_T<float>(h, blk, ncol, X, Y, m, a, b, a0);
  h->err = "cx_chebyshev_filter: bad prec";
  return CX_ERR_ARG;
}

cx_status cx_sync(cx_handle h) {
  if (!h) return CX_ERR_ARG;
  CX_TRY_CUDA(h, cudaStreamSynchronize(h->stream));
  return CX_OK;
}

cx_status cx_timer_start(cx_handle h) {
  if (!h) return CX_ERR_ARG;
  CX_TRY_CUDA(h, cudaEventRecord(h->tev0, h->stream));
  return CX_OK;
}

cx_status cx_timer_stop(cx_handle h, double* ms) {
  if (!h || !ms) return CX_ERR_ARG;
  CX_TRY_CUDA(h, cudaEventRecord(h->tev1, h->stream));
  CX_TRY_CUDA(h, cudaEventSynchronize(h->tev1));
  float f = 0;
  CX_TRY_CUDA(h, cudaEventElapsedTime(&f, h->tev0, h->tev1));
  *ms = f;
  return CX_OK;
}

cx_status cx_profile_stencil(cx_handle h, int32_t enable) {
  if (!h) return CX_ERR_ARG;
  h->prof = enable != 0;
  h->prof_launches = 0;
  h->prof_ms = 0;
  h->prof_apply_ms = 0;
  h->prof_contract_ms = 0;
  h->prof_bytes = 0;
  return CX_OK;
}

cx_status cx_profile_read_apply(cx_handle h, double* apply_ms) {
  if (!h || !apply_ms) return CX_ERR_ARG;
  *apply_ms = h->prof_apply_ms;
  return CX_OK;
}

cx_status cx_set_nl_kernels(cx_handle h, int32_t tensor_cores) {
  if (!h) return CX_ERR_ARG;
  if (tensor_cores && !h->nltc_contract) {
    h->err = "cx_set_nl_kernels: the tensor-core projector kernels need at most 8 images per atom";
    return CX_ERR_ARG;
  }
  h->use_nltc = tensor_cores != 0;
  return CX_OK;
}

cx_status cx_profile_read_contract(cx_handle h, double* contract_ms) {
  if (!h || !contract_ms) return CX_ERR_ARG;
  *contract_ms = h->prof_contract_ms;
  return CX_OK;
}

cx_status cx_profile_read(cx_handle h, int64_t* launches, double* total_ms, double* bytes) {
  if (!h) return CX_ERR_ARG;
  if (launches) *launches = h->prof_launches;
  if (total_ms) *total_ms = h->prof_ms;
  if (bytes) *bytes = h->prof_bytes;
  return CX_OK;
}

cx_status cx_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return CX_ERR_ARG;
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) { g_create_err = std::string("cx_host_register: ") + cudaGetErrorString(e); return CX_ERR_CUDA; }
  return CX_OK;
}

cx_status cx_host_unregister(void* ptr) {
  if (!ptr) return CX_ERR_ARG;
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) { g_create_err = std::string("cx_host_unregister: ") + cudaGetErrorString(e); return CX_ERR_CUDA; }
  return CX_OK;
}

cx_status cx_stencil_config(cx_handle h, int32_t* rows_per_thread, int32_t* ring_depth, int32_t* tuned, char* log, int32_t log_bytes) {
  if (!h || !rows_per_thread || !ring_depth || !tuned) return CX_ERR_ARG;
  *rows_per_thread = h->tma_rpt;
  *ring_depth = h->tma_depth;
  *tuned = h->tma_tuned ? 1 : 0;
  if (log && log_bytes > 0) {
    const size_t n = std::min((size_t)log_bytes - 1, h->tma_tuning.size());
    std::copy(h->tma_tuning.begin(), h->tma_tuning.begin() + n, log);
    log[n] = 0;
  }
  return CX_OK;
}

cx_status cx_launch_count(cx_handle h, int64_t* count, int32_t reset) {
  if (!h) return CX_ERR_ARG;
  if (count) *count = h->launches;
  if (reset) h->launches = 0;
  return CX_OK;
}

}  // extern "C"
