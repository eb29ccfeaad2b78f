// cx_hpsi_noalloc: H*psi on caller-owned device buffers without any device allocation.
//
// Some callers cannot let a library call cudaMalloc: their device memory is owned by another
// allocator (a host framework's caching allocator that accounts for every byte, or a MEX session
// that must leave nothing allocated behind when MATLAB interrupts it).  This entry point serves
// them.  The caller passes the input block X and the output Y as device pointers; the only extra
// device memory the product needs -- the per-state projector coefficients of the Kleinman-Bylander
// term and a few small descriptors -- lives in the fixed array g_noalloc_scratch below, which is
// part of the library's device image.  Every GPU that loads the library holds that array (16 MiB)
// until the process exits.
//
// The array's name is only a host-side stand-in in host code, so the first call on each device
// looks up its device address with cudaGetSymbolAddress (with that device current) and keeps it;
// that first call should therefore come before any stream capture.  All calls share the one array
// and it keeps the contents of the last call: every byte a call reads is written earlier by the
// same call (the descriptors by a copy, the projector coefficients by the contraction kernel), so
// nothing needs clearing, but two calls whose work overlaps on the GPU (different handles or
// threads at the same time) race on it.  Each call waits for its own work before returning.
#include <cstring>
#include <mutex>

#include "cx_common.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;   // 16 MiB per device
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
cx_status scratch_address(cx_handle h, int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) { h->err = "cx_hpsi_noalloc: device ordinal out of range"; return CX_ERR_ARG; }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      h->err = std::string("cx_hpsi_noalloc: cudaGetSymbolAddress of the scratch array failed: ") + cudaGetErrorString(e);
      return CX_ERR_CUDA;
    }
    g_scratch_ptr[dev] = (unsigned char*)p;
  }
  *out = g_scratch_ptr[dev];
  return CX_OK;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename R>
cx_status hpsi_noalloc_T(cx_handle h, int blk, int ncol, const void* X, void* Y, unsigned char* scratch) {
  using namespace cx;
  const int nseg = std::max(1, h->nl.nseg);
  // layout of the scratch for this call
  const size_t o_blk = 0;
  const size_t o_tab = o_blk + align256(sizeof(BlockDev<R>));
  const size_t o_scal = o_tab + align256(sizeof(int2) * (size_t)ncol);
  const size_t o_ph = o_scal + align256(sizeof(StepScalars));
  const size_t o_cp = o_ph + align256(sizeof(double2) * (size_t)nseg);
  const size_t need = o_cp + align256(sizeof(cplx<R>) * (size_t)ncol * nseg * kAngMax);
  if (need > kNoAllocScratchBytes) {
    const size_t per_col = sizeof(cplx<R>) * (size_t)nseg * kAngMax + sizeof(int2);
    const size_t fixed = o_cp - sizeof(int2) * (size_t)ncol;
    h->err = "cx_hpsi_noalloc: " + std::to_string(ncol) + " columns need " + std::to_string(need) +
             " B of scratch but the static scratch holds " + std::to_string(kNoAllocScratchBytes) +
             " B; at most " + std::to_string((kNoAllocScratchBytes - fixed - 2048) / per_col) +
             " columns per call for this operator";
    return CX_ERR_ARG;
  }
  BlockDev<R>* d_blk = (BlockDev<R>*)(scratch + o_blk);
  int2* d_tab = (int2*)(scratch + o_tab);
  StepScalars* d_scal = (StepScalars*)(scratch + o_scal);
  double2* d_ph = (double2*)(scratch + o_ph);
  cplx<R>* cprime = (cplx<R>*)(scratch + o_cp);

  std::vector<BlockDev<R>> bd;
  std::vector<cplx<R>*> p0{(cplx<R>*)X}, p1{(cplx<R>*)Y};
  make_block_devs<R>(h, p0, p1, std::vector<int>{blk}, bd);
  bd[0].Ns = ncol;
  std::vector<int2> tab(ncol);
  for (int i = 0; i < ncol; ++i) tab[i] = make_int2(0, i);
  const StepScalars one{1.0, 0.0, 0.0, 0.0};
  std::vector<double2> ph = segment_phases(h, h->blocks[blk]);
  if (ph.empty()) ph.push_back(make_double2(1, 0));
  cudaStream_t st = h->stream;
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_blk, bd.data(), sizeof(BlockDev<R>), cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_tab, tab.data(), sizeof(int2) * tab.size(), cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_scal, &one, sizeof(one), cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_ph, ph.data(), sizeof(double2) * ph.size(), cudaMemcpyHostToDevice, st));
  NonlocalDev nl = h->nl;
  nl.seg_phase = d_ph;
  nl.seg_phase32 = nullptr;
  nl.node_wchi = sizeof(R) == 4 ? h->d_node_wchi32 : h->d_node_wchi64;
  nl.ent_chi = sizeof(R) == 4 ? h->d_ent_chi32 : h->d_ent_chi64;
  const bool nonlocal = nl.nseg > 0;
  if (nonlocal) {
    CX_TRY_CUDA(h, launch_nl_contract<R>(h->g, d_blk, d_tab, ncol, 0, nl, cprime, st));
    h->launches++;
  }
  CX_TRY_CUDA(h, launch_cheb_step<R>(h->g, h->coef, d_blk, d_scal, 1, d_tab, ncol, 0, false, nonlocal ? &nl : nullptr, cprime, st));
  h->launches++;
  // the host-side descriptors above must outlive the copies, and the caller may reuse the
  // scratch right after: wait for this call's work
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  return CX_OK;
}

}  // namespace

extern "C" cx_status cx_hpsi_noalloc(cx_handle h, int32_t blk, int32_t ncol, const void* X_dev, void* Y_dev, int32_t prec) {
  if (!h) return CX_ERR_ARG;
  if (!X_dev || !Y_dev || X_dev == Y_dev) { h->err = "cx_hpsi_noalloc: need distinct device pointers X and Y"; return CX_ERR_ARG; }
  if (blk < 0 || blk >= h->nblk) { h->err = "cx_hpsi_noalloc: block index out of range (call cx_set_blocks first)"; return CX_ERR_STATE; }
  if (ncol < 1 || ncol > 65535) { h->err = "cx_hpsi_noalloc: ncol must be in 1..65535"; return CX_ERR_ARG; }
  if (prec != CX_PREC_FP64 && prec != CX_PREC_MIXED) { h->err = "cx_hpsi_noalloc: bad prec"; return CX_ERR_ARG; }
  int prev = -1;
  CX_TRY_CUDA(h, cudaGetDevice(&prev));
  if (prev != h->dev) CX_TRY_CUDA(h, cudaSetDevice(h->dev));
  unsigned char* scratch = nullptr;
  cx_status s = scratch_address(h, h->dev, &scratch);
  if (s == CX_OK)
    s = prec == CX_PREC_FP64 ? hpsi_noalloc_T<double>(h, blk, ncol, X_dev, Y_dev, scratch)
                             : hpsi_noalloc_T<float>(h, blk, ncol, X_dev, Y_dev, scratch);
  if (prev != h->dev) cudaSetDevice(prev);
  return s;
}
