// Internal definitions of libcyclix_gpu.so (not part of the C-ABI).
#pragma once

#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cyclix_gpu.h"

namespace cx {

struct ScfState;                  // SCF run between cx_scf_init and cx_scf_finish (cx_scf.cu)

constexpr int kMaxFDn = 8;

// ---------------------------------------------------------------- complex helpers
template <typename R> struct C2;
template <> struct C2<float> { using T = float2; };
template <> struct C2<double> { using T = double2; };
template <typename R> using cplx = typename C2<R>::T;

template <typename R> __host__ __device__ __forceinline__ cplx<R> mk(R x, R y) { cplx<R> c; c.x = x; c.y = y; return c; }
template <typename V> __host__ __device__ __forceinline__ V cadd(V a, V b) { V c; c.x = a.x + b.x; c.y = a.y + b.y; return c; }
template <typename V> __host__ __device__ __forceinline__ V csub(V a, V b) { V c; c.x = a.x - b.x; c.y = a.y - b.y; return c; }
template <typename V, typename R> __host__ __device__ __forceinline__ V cscale(V a, R s) { V c; c.x = a.x * s; c.y = a.y * s; return c; }
template <typename V> __host__ __device__ __forceinline__ V cmul(V a, V b) {
  V c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
template <typename V> __host__ __device__ __forceinline__ V cmulconj(V a, V b) {  // conj(a) * b
  V c; c.x = a.x * b.x + a.y * b.y; c.y = a.x * b.y - a.y * b.x; return c;
}
// acc += s * a  (s real)
template <typename V, typename R> __host__ __device__ __forceinline__ void cfma(V& acc, R s, V a) {
  acc.x = fma(s, a.x, acc.x); acc.y = fma(s, a.y, acc.y);
}

// ---------------------------------------------------------------- operator description
// Coefficients of the 1-D stencils (index q = 0..FDn, symmetric / antisymmetric parts).
struct StencilCoef {
  double cr2[kMaxFDn + 1];   // w2[q] / dx^2
  double cr1[kMaxFDn + 1];   // w1[q] / dx          (times 1/r_i per radial row)
  double ct2[kMaxFDn + 1];   // w2[q] / dy^2        (times theta scale per radial row)
  double ct1[kMaxFDn + 1];   // -2 tau w1[q] / dy   (helical cross term, theta part)
  double cz2[kMaxFDn + 1];   // w2[q] / dz^2
  double cz1[kMaxFDn + 1];   // w1[q] / dz          (helical cross term, z part)
};

// Per-block data the kernels read (device array, one entry per block).
template <typename R> struct BlockDev {
  cplx<R>* buf[2];           // psi and work buffers, N x Ns each (column-major)
  const double* veff;        // N (the block's spin channel)
  double2 ph_tl, ph_tr;      // theta wrap phases exp(-+ i k2 L2) (1 when k2 == 0)
  double2 ph_zl, ph_zr;      // z wrap phases exp(-+ i k3 L3)
  int32_t Ns;
  int32_t state0;            // first global state index of this block
  int32_t veff_spin;         // spin channel (selects the Veff map of the TMA path)
  int32_t pad;
};

// Chebyshev step scalars of one block for one degree: out = alpha*(H*in - c*in) + beta*xprev
struct StepScalars { double alpha, c, beta, pad; };

struct NonlocalDev {
  int32_t n_atm, nseg, nnode;                // atoms, (atom,image) segments, total ball nodes
  const int32_t* atom_node_ptr;              // n_atm+1, nodes of atom J (all its images)
  const int32_t* node_pos;                   // nnode, 0-based grid index
  const int32_t* node_seg;                   // nnode, global segment id
  const void* node_wchi;                     // nnode x 4(angmax) real: W * Chi (R)
  const int32_t* atom_seg_ptr;               // n_atm+1, segments of atom J
  const double* gamma;                       // n_atm x angmax
  const int32_t* angnum;                     // n_atm
  const int32_t* row_ptr;                    // N+1, entries covering grid point p
  const int32_t* ent_seg;                    // entries: segment id
  const void* ent_chi;                       // entries x angmax real: Chi
  const double2* seg_phase;                  // nblk x nseg: exp(i k.(R_J - R_img)) per block
  const float2* seg_phase32;                 // the same in float for the complex64 path (or null)
};

constexpr int kAngMax = 4;   // l <= 1 projectors: (lmax+1)^2 = 4 columns per atom at most

struct GridDev {
  int32_t Nx, Ny, Nz, N;
  int32_t FDn, helical, BCy, BCz;
  double xin, dx, twist;
};

// ---------------------------------------------------------------- kernels (cx_stencil.cu)
template <typename R>
cudaError_t launch_cheb_step(const GridDev& g, const StencilCoef& coef, const BlockDev<R>* blocks,
                             const StepScalars* scal, int nblk, const int2* state_tab, int nstates,
                             int in_sel, bool use_xprev, const NonlocalDev* nl, const cplx<R>* cprime,
                             cudaStream_t st);
// 32-point row chunks touched by projector balls, with the dense Chi of each chunk
// (32 points x K = 4 x the chunk's segments, stored [K][32], zero outside the balls).
struct ChunkTables {
  int32_t nchunks, kmax;
  const int32_t* p0;          // first grid point of the chunk
  const int32_t* seg_ptr;     // nchunks + 1
  const int32_t* segs;        // segment ids of each chunk
  const int64_t* chi_ptr;     // offset of the chunk's Chi block (elements)
  const void* chi;            // float or double, per precision
};
template <typename R>
cudaError_t launch_nl_apply(const GridDev& g, const BlockDev<R>* blocks, const StepScalars* scal, const int2* state_tab, int nstates,
                            int out_sel, const ChunkTables& ct, const cplx<R>* cprime, int nseg, cudaStream_t st);
template <typename R>
cudaError_t launch_nl_contract(const GridDev& g, const BlockDev<R>* blocks, const int2* state_tab, int nstates,
                               int in_sel, const NonlocalDev& nl, cplx<R>* cprime, cudaStream_t st);

// ---------------------------------------------------------------- tensor-core projector term (cx_nl_tc.cu)
// Device copies of the B-operand images (hi / lo tf32 parts of W Chi per atom and of Chi per
// chunk in the tcgen05 core-matrix layout), made once per operator.
struct NlTcImages {
  const int64_t* ct_ptr = nullptr;   // n_atm: float offset of the atom's image
  const float* ct_img = nullptr;
  const int64_t* ap_ptr = nullptr;   // nchunks: float offset of the chunk's image
  const float* ap_img = nullptr;
};
// host: the images (false when an atom has more than 8 images: the CUDA-core contraction is used)
bool nl_tc_contract_images(const std::vector<int32_t>& atom_node_ptr, const std::vector<int32_t>& node_seg,
                           const std::vector<int32_t>& atom_seg_ptr, const std::vector<double>& node_wchi, std::vector<int64_t>& ptr,
                           std::vector<float>& img);
void nl_tc_apply_images(const std::vector<int32_t>& cseg_ptr, const std::vector<int64_t>& cchi_ptr, const std::vector<double>& cchi,
                        std::vector<int64_t>& ptr, std::vector<float>& img);
cudaError_t launch_nl_contract_tc(const GridDev& g, const BlockDev<float>* blocks, const int2* state_tab, int nstates, int in_sel,
                                  const NonlocalDev& nl, const NlTcImages& im, float2* cprime, int* status, cudaStream_t st);
cudaError_t launch_nl_apply_tc(const GridDev& g, const BlockDev<float>* blocks, const StepScalars* scal, const int2* state_tab,
                               int nstates, int out_sel, const ChunkTables& ct, const NlTcImages& im, const float2* cprime, int nseg,
                               int* status, cudaStream_t st);

// ---------------------------------------------------------------- TMA path (cx_stencil_tma.cu)
// Device arrays of tensor maps used by one launch of the TMA kernel.
struct TmaMapSet {
  const void* xmaps;         // [block][buffer] complex64 X maps (staged tile rows)
  const void* hmaps;         // [block][buffer] complex64 theta-halo maps
  const void* omaps;         // [block][buffer] complex64 output-tile maps
  const void* vmaps;         // [spin] float Veff maps
};
bool tma_eligible(const GridDev& g, int elem_bytes);
cudaError_t launch_cheb_step_tma(const GridDev& g, const StencilCoef& coef, const BlockDev<float>* blocks, const StepScalars* scal,
                                 const int2* state_tab, int nstates, int in_sel, bool use_xprev, const TmaMapSet& maps, int* status,
                                 cudaStream_t st, int rpt = 0, int depth = 0);
// (rows per thread, prefetch depth) configurations of the TMA kernel for this grid (autotuner)
int tma_candidates(const GridDev& g, int* rpt, int* depth, int cap);

}  // namespace cx

// ---------------------------------------------------------------- the handle
// Resources of one concurrent Rayleigh-Ritz worker (its own stream, library handles and
// workspaces), kept by the handle between eigSolver calls.
struct cx_rr_worker {
  cudaStream_t stream = nullptr;
  cublasHandle_t cublas = nullptr;
  cusolverDnHandle_t cusolver = nullptr;
  cusolverDnParams_t params = nullptr;
  void* d_ws = nullptr; size_t ws_bytes = 0;
  void* h_ws = nullptr; size_t hws_bytes = 0;
  void* d_rr = nullptr; size_t rr_bytes = 0;
};

struct cx_handle_s {
  std::string err;
  int dev = 0;
  cudaStream_t stream = nullptr;
  cublasHandle_t cublas = nullptr;
  cusolverDnHandle_t cusolver = nullptr;
  cusolverDnParams_t cusolver_params = nullptr;

  // grid
  cx_grid grid{};
  cx::GridDev g{};
  cx::StencilCoef coef{};
  double w1[cx::kMaxFDn + 1] = {};   // S.w1, first-derivative weights (gradients of the GGA potential)
  std::vector<double> W;      // host copy
  double* d_W = nullptr;
  float* d_W32 = nullptr;                            // float copy of W for the complex64 kernels
  int nspin = 1;
  double* d_veff = nullptr;   // N x nspin

  // nonlocal
  cx::NonlocalDev nl{};
  std::vector<void*> nl_allocs;
  std::vector<int32_t> seg_atom;                     // segment -> atom
  std::vector<double> seg_coord;                     // nseg x 3
  std::vector<double> atom_pos;                      // n_atm x 3
  void* d_node_wchi32 = nullptr;
  void* d_ent_chi32 = nullptr;
  void* d_node_wchi64 = nullptr;
  void* d_ent_chi64 = nullptr;
  double2* d_seg_phase = nullptr;
  float2* d_seg_phase32 = nullptr;

  // blocks
  int nblk = 0;
  int prec = CX_PREC_FP64;
  std::vector<cx_block> blocks;
  std::vector<int32_t> state0;                       // first global state per block
  int nstates = 0;
  std::vector<void*> bufs;                           // 2 per block
  void* d_blocks = nullptr;                          // BlockDev<R>[nblk] of the current precision
  int2* d_state_tab = nullptr;
  void* d_cprime = nullptr;                          // nstates x nseg x 4 complex (current precision)
  cx::StepScalars* d_scal = nullptr;                 // npl_max x nblk
  int scal_cap = 0;
  std::vector<void*> ubgv;                           // per block N complex128 (upper-bound vectors)
  int where[1] = {0};                                // which buffer holds psi per block (same for all)
  std::vector<int> psi_sel;                          // per block: 0/1 buffer index holding psi

  // subspace workspace
  void* d_ws = nullptr; size_t ws_bytes = 0;
  void* h_ws = nullptr; size_t hws_bytes = 0;
  void* d_stage = nullptr; size_t stage_bytes = 0;   // host-transfer staging (complex128)
  void* d_rr = nullptr; size_t rr_bytes = 0;         // Rayleigh-Ritz matrices
  void* d_lz = nullptr; size_t lz_bytes = 0;         // Lanczos vectors and scalars
  void* d_misc = nullptr; size_t misc_bytes = 0;     // column norms, permutations, status
  void* d_pois = nullptr; size_t pois_bytes = 0;     // Poisson (AAR) vectors
  void* d_scf = nullptr; size_t scf_bytes = 0;       // SCF state (density, potentials, mixing history)
  cx::ScfState* scf = nullptr;                       // loop state of the SCF run in progress

  // TMA path (complex64): float Veff, per-point projector entry start / count, tensor maps
  float* d_veff32 = nullptr;
  cx::ChunkTables chunks32{}, chunks64{};           // projector chunks (complex64 / complex128 Chi)
  cx::NlTcImages nltc{};                             // tensor-core projector operands (complex64)
  bool nltc_contract = false, nltc_apply = false;    // images present: the tcgen05 kernels are used
  bool use_nltc = false;                             // cx_set_nl_kernels: the tcgen05 projector kernels
  void* d_fmaps = nullptr;                           // [nspin] Veff maps
  void* d_maps = nullptr;                            // block buffers: [nblk][2] X, halo and output maps
  cx::TmaMapSet tma_main{};
  bool tma_ok = false;                               // operator eligible for the TMA kernel
  int* d_status = nullptr;
  bool use_tma = true;
  int tma_rpt = 0, tma_depth = 0;                    // TMA kernel configuration (0: default rule)
  bool tma_tuned = false;                            // the autotuner has chosen it for this handle
  std::string tma_tuning;                            // candidates and times of the last tuning (ms)

  // profiling
  bool prof = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, tev0 = nullptr, tev1 = nullptr, cev = nullptr;
  cudaEvent_t eig_ev[3] = {nullptr, nullptr, nullptr};   // eigSolver parts (start, after filter and H X, end)
  double last_filter_ms = 0, last_rr_ms = 0;
  int64_t prof_launches = 0;
  double prof_ms = 0, prof_bytes = 0, prof_apply_ms = 0, prof_contract_ms = 0;
  int64_t launches = 0;
  int64_t eig_fallbacks = 0;                         // subspace eigensolves that needed the general solver
  int64_t eig_restarts = 0;                          // similarity restarts of the eigenvector refinement
  int64_t eig_hermitian = 0;                         // subspace eigensolves answered by the Hermitian part
  int restart_fail_streak = 0;                       // blocks in a row whose restarts ended in the general solver
  int* rr_tier = nullptr;                            // per block: the refinement tier that succeeded last (shared by workers)
  int rr_tier_n = 0;
  std::vector<cx_rr_worker> rr_workers;              // concurrent Rayleigh-Ritz of the blocks
};

#define CX_TRY_CUDA(h, expr)                                                                 \
  do {                                                                                       \
    cudaError_t _e = (expr);                                                                 \
    if (_e != cudaSuccess) {                                                                 \
      (h)->err = std::string(#expr) + ": " + cudaGetErrorString(_e);                          \
      return _e == cudaErrorMemoryAllocation ? CX_ERR_NOMEM : CX_ERR_CUDA;                   \
    }                                                                                        \
  } while (0)
