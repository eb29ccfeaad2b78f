// Host-side helpers shared by the translation units of libcyclix_gpu.so.
#pragma once
#include <vector>

#include "cx_internal.h"

// host complex128 (interleaved) <-> device buffer in the given precision
cx_status cx_host_to_dev(cx_handle h, const double* host, void* dev, size_t n_complex, int prec);
cx_status cx_dev_to_host(cx_handle h, const void* dev, double* host, size_t n_complex, int prec);
// releases the workspaces owned by cx_linalg.cu / cx_poisson.cu
void cx_free_extra(cx_handle h);

namespace cx {

template <typename R>
cx_status make_block_devs(cx_handle h, const std::vector<cplx<R>*>& b0, const std::vector<cplx<R>*>& b1,
                          const std::vector<int>& blk_ids, std::vector<BlockDev<R>>& out);
std::vector<double2> segment_phases(cx_handle h, const cx_block& B);
void cheb_scalars(int m, double a, double b, double a0, std::vector<StepScalars>& out, int stride, int col);

template <typename R>
cx_status fused_step(cx_handle h, const BlockDev<R>* d_blocks, const StepScalars* d_scal, int nblk, const int2* d_state_tab,
                     int nstates, int in_sel, bool use_xprev, cplx<R>* cprime, bool nonlocal, double bytes,
                     const void* maps = nullptr);
template <typename R>
cx_status filter_blocks(cx_handle h, const BlockDev<R>* d_blocks, int nblk, const int2* d_state_tab, int nstates,
                        size_t total_elems, int sel0, int m, const std::vector<double>& a, const std::vector<double>& b,
                        const std::vector<double>& a0, cplx<R>* cprime, int* sel_out, const void* maps = nullptr);
// tensor maps of one complex64 buffer of Ns states / of a 4-byte grid field (cx_stencil_tma.cu)
cx_status make_buffer_maps(cx_handle h, const void* base, int Ns, struct CUtensorMap_st* xmap, struct CUtensorMap_st* hmap,
                           struct CUtensorMap_st* omap);
cx_status make_field_map(cx_handle h, const void* base, bool is_int, struct CUtensorMap_st* out);
// build the X / output maps of device buffers p0/p1 of a block set into a new device array and
// fill the block part of *set (the field maps of the handle complete it)
cx_status build_maps(cx_handle h, const std::vector<const void*>& p0, const std::vector<const void*>& p1,
                     const std::vector<int>& Ns, void** d_maps, TmaMapSet* set);
// AAR Poisson solve on device vectors (cx_poisson.cu)
cx_status poisson_dev(cx_handle h, const double* d_f, double* d_phi, double tol, int32_t maxit, int32_t use_guess, int32_t* iters,
                      double* relres_out);
cudaError_t launch_pinv_solve(double* io, int m, cudaStream_t st);
// releases the SCF loop state (cx_scf.cu)
void scf_state_free(cx_handle h);
// FP64 Rayleigh quotients of the device-resident psi (cx_linalg.cu)
cx_status refine_eigenvalues(cx_handle h, double* EigVal);
// tensor-core (tcgen05) Rayleigh-Ritz products of the complex64 path (cx_tcgen05.cu):
// C (n x m complex128, leading dimension ldc) = X^H (w .* Y), w optional; Z (N x m) = X C with C complex128
cx_status tc_gram(cx_handle h, const float2* X, const float2* Y, const float* w, int N, int n, int m, double2* C, int ldc);
size_t tc_rot_image_floats(int n, int m);
cx_status tc_rotate(cx_handle h, const float2* X, const double2* C, int N, int n, int m, float2* Z, float* img);
// status flag of the TMA pipeline: CX_OK, or CX_ERR_CUDA with a message when a CTA timed out
cx_status check_pipeline_status(cx_handle h);

}  // namespace cx
