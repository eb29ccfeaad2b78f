// Atomic forces on the GPU: the nonlocal term of src/atomicForce.m:254-300 over the device-resident
// psi of every block, and the Cartesian gradient of a grid field (the S.grad_1..3 products of
// src/atomicForce.m that the local and correction terms take of phi and V_c).  The per-point
// arithmetic is in cx_force_point.h; the products psi^H [W Ck | W D Ck] are one ZGEMM per block.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cx_common.h"
#include "cx_force_point.h"

namespace cx {

static_assert(force::kCols == kAngMax, "force fields hold the projector kernels' columns per atom");
static_assert(force::kMaxFDn == kMaxFDn, "force stencils cover every supported FD order");
static_assert(sizeof(force::Cd) == sizeof(double2), "complex128 layout");

__global__ void k_force_fields(int N, int C, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ ent_seg,
                               const double* __restrict__ ent_chi, const force::SegForce* __restrict__ seg, force::Cd* Ck,
                               force::Cd* R1, force::Cd* R2) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
    force::force_fields_point(p, (size_t)N, C, row_ptr, ent_seg, ent_chi, seg, Ck, R1, R2);
}

__global__ void k_force_grad(int N, int C, force::ForceGrid g, const force::Cd* __restrict__ Ck, const force::Cd* __restrict__ R1,
                             const force::Cd* __restrict__ R2, const double* __restrict__ W, force::Cd* __restrict__ out) {
  const size_t total = (size_t)N * C;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(idx / N), p = (int)(idx % N);
    force::force_grad_point(p, (size_t)N, C, c, g, Ck, R1, R2, W, out);
  }
}

__global__ void k_real_grad(int N, force::ForceGrid g, const double* __restrict__ u, double* __restrict__ D) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) force::real_grad_point(p, g, u, D);
}

__global__ void k_widen(const float2* __restrict__ a, double2* __restrict__ b, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = make_double2(a[i].x, a[i].y);
}

static unsigned grid_for(size_t n) { return (unsigned)std::min<size_t>(152 * 16, (n + 255) / 256); }

// grid part of the force data (the Bloch phases are set per block)
static force::ForceGrid force_grid(cx_handle h) {
  force::ForceGrid g{};
  g.Nx = h->g.Nx; g.Ny = h->g.Ny; g.Nz = h->g.Nz; g.FDn = h->g.FDn;
  g.xin = h->grid.xin; g.dx = h->grid.dx; g.dy = h->grid.dy; g.dz = h->grid.dz; g.twist = h->grid.twist;
  g.cL2 = std::cos(h->grid.L2);
  g.sL2 = std::sin(h->grid.L2);
  for (int q = 0; q <= h->g.FDn; ++q) g.w1[q] = h->w1[q];
  return g;
}

// device buffers of one cx_nonlocal_force call
struct ForceScratch {
  void* base = nullptr;
  ~ForceScratch() { if (base) cudaFree(base); }
};

}  // namespace cx

using namespace cx;

extern "C" cx_status cx_nonlocal_force(cx_handle h, const double* occ, const double* wkpt, double occfac, double* F) {
  if (!h) return CX_ERR_ARG;
  if (!occ || !wkpt || !F) { h->err = "cx_nonlocal_force: occ, wkpt and F are required"; return CX_ERR_ARG; }
  if (h->nblk < 1) { h->err = "cx_nonlocal_force: call cx_set_blocks (and cx_set_psi) first"; return CX_ERR_STATE; }
  const int N = h->g.N, nat = h->nl.n_atm, nseg = h->nl.nseg, C = kAngMax * nat;
  std::fill(F, F + 3 * (size_t)std::max(nat, 0), 0.0);
  if (nat == 0 || nseg == 0) return CX_OK;
  const cudaStream_t st = h->stream;
  int ns_max = 0;
  for (const cx_block& B : h->blocks) ns_max = std::max(ns_max, (int)B.Ns);
  // projector fields (3 N C), W-weighted fields and gradients (4 N C), widened complex64 psi,
  // products (Ns x 4C), segment table
  const size_t nc = (size_t)N * C;
  const size_t b_fields = 3 * nc * 16, b_out = 4 * nc * 16, b_psi = h->prec == CX_PREC_FP64 ? 0 : (size_t)N * ns_max * 16,
               b_P = (size_t)ns_max * 4 * C * 16, b_seg = (size_t)nseg * sizeof(force::SegForce);
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  ForceScratch sc;
  if (cudaMalloc(&sc.base, up(b_fields) + up(b_out) + up(b_psi) + up(b_P) + up(b_seg)) != cudaSuccess) {
    cudaGetLastError();
    h->err = "cx_nonlocal_force: device allocation failed";
    return CX_ERR_NOMEM;
  }
  char* q = (char*)sc.base;
  force::Cd* Ck = (force::Cd*)q;
  force::Cd* R1 = Ck + nc;
  force::Cd* R2 = R1 + nc;
  q += up(b_fields);
  force::Cd* out = (force::Cd*)q;
  q += up(b_out);
  double2* psi64 = (double2*)q;
  q += up(b_psi);
  force::Cd* d_P = (force::Cd*)q;
  q += up(b_P);
  force::SegForce* d_seg = (force::SegForce*)q;
  // gamma of every column (zero beyond the atom's angnum)
  std::vector<double> gamma((size_t)nat * kAngMax);
  CX_TRY_CUDA(h, cudaMemcpyAsync(gamma.data(), h->nl.gamma, gamma.size() * 8, cudaMemcpyDeviceToHost, st));
  const double L2 = h->grid.L2, L3 = h->grid.L3, tau = h->grid.twist;
  std::vector<force::SegForce> seg(nseg);
  std::vector<force::Cd> P((size_t)ns_max * 4 * C);
  int off = 0;
  for (int b = 0; b < h->nblk; ++b) {
    const cx_block& B = h->blocks[b];
    const int Ns = B.Ns;
    const double* k = B.kpt_vec;
    force::segment_table(nseg, h->seg_atom.data(), h->seg_coord.data(), h->atom_pos.data(), k, L2, L3, tau, seg.data());
    force::ForceGrid g = force_grid(h);
    force::set_bloch_phases(g, k, L2, L3);
    CX_TRY_CUDA(h, cudaMemcpyAsync(d_seg, seg.data(), b_seg, cudaMemcpyHostToDevice, st));
    k_force_fields<<<grid_for(N), 256, 0, st>>>(N, C, h->nl.row_ptr, h->nl.ent_seg, (const double*)h->d_ent_chi64, d_seg, Ck, R1, R2);
    k_force_grad<<<grid_for(nc), 256, 0, st>>>(N, C, g, Ck, R1, R2, h->d_W, out);
    h->launches += 2;
    const void* psi = h->bufs[2 * b + h->psi_sel[0]];
    if (h->prec != CX_PREC_FP64) {
      k_widen<<<grid_for((size_t)N * Ns), 256, 0, st>>>((const float2*)psi, psi64, (size_t)N * Ns);
      h->launches++;
      psi = psi64;
    }
    CX_TRY_CUDA(h, cudaGetLastError());
    const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
    if (cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH) != CUBLAS_STATUS_SUCCESS ||
        cublasZgemm(h->cublas, CUBLAS_OP_C, CUBLAS_OP_N, Ns, 4 * C, N, &one, (const cuDoubleComplex*)psi, N,
                    (const cuDoubleComplex*)out, N, &zero, (cuDoubleComplex*)d_P, Ns) != CUBLAS_STATUS_SUCCESS) {
      h->err = "cx_nonlocal_force: cublasZgemm failed";
      return CX_ERR_LIB;
    }
    CX_TRY_CUDA(h, cudaMemcpyAsync(P.data(), d_P, (size_t)Ns * 4 * C * 16, cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    force::force_accumulate(Ns, nat, P.data(), occ + off, gamma.data(), occfac * 2.0 * wkpt[b], F);
    off += Ns;
  }
  return CX_OK;
}

extern "C" cx_status cx_gradient(cx_handle h, const double* f, double* Df) {
  if (!h) return CX_ERR_ARG;
  if (!f || !Df) { h->err = "cx_gradient: f and Df are required"; return CX_ERR_ARG; }
  if (h->grid.BCy != 0 || h->grid.BCz != 0) { h->err = "cx_gradient: theta and z must be periodic (BCy = BCz = 0)"; return CX_ERR_ARG; }
  const int N = h->g.N;
  const cudaStream_t st = h->stream;
  ForceScratch sc;
  if (cudaMalloc(&sc.base, (size_t)N * 8 * 4) != cudaSuccess) {
    cudaGetLastError();
    h->err = "cx_gradient: device allocation failed";
    return CX_ERR_NOMEM;
  }
  double* d_u = (double*)sc.base;
  double* d_D = d_u + N;
  const force::ForceGrid g = force_grid(h);
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_u, f, (size_t)N * 8, cudaMemcpyHostToDevice, st));
  k_real_grad<<<grid_for(N), 256, 0, st>>>(N, g, d_u, d_D);
  h->launches++;
  CX_TRY_CUDA(h, cudaGetLastError());
  CX_TRY_CUDA(h, cudaMemcpyAsync(Df, d_D, (size_t)N * 8 * 3, cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  return CX_OK;
}

extern "C" cx_status cx_field_projections(cx_handle h, const double* f, int32_t nvec, const double* A, double* out) {
  if (!h) return CX_ERR_ARG;
  if (!f || (nvec > 0 && (!A || !out)) || nvec < 0) { h->err = "cx_field_projections: f, A and out are required, nvec >= 0"; return CX_ERR_ARG; }
  if (h->grid.BCy != 0 || h->grid.BCz != 0) { h->err = "cx_field_projections: theta and z must be periodic (BCy = BCz = 0)"; return CX_ERR_ARG; }
  if (nvec == 0) return CX_OK;
  const int N = h->g.N;
  const cudaStream_t st = h->stream;
  ForceScratch sc;
  const size_t n_f = (size_t)N, n_D = 3 * (size_t)N, n_A = (size_t)nvec * N, n_o = 3 * (size_t)nvec;
  if (cudaMalloc(&sc.base, (n_f + n_D + n_A + n_o) * 8) != cudaSuccess) {
    cudaGetLastError();
    h->err = "cx_field_projections: device allocation failed";
    return CX_ERR_NOMEM;
  }
  double* d_f = (double*)sc.base;
  double* d_D = d_f + n_f;
  double* d_A = d_D + n_D;
  double* d_o = d_A + n_A;
  const force::ForceGrid g = force_grid(h);
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_f, f, n_f * 8, cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(d_A, A, n_A * 8, cudaMemcpyHostToDevice, st));
  k_real_grad<<<grid_for(N), 256, 0, st>>>(N, g, d_f, d_D);
  h->launches++;
  CX_TRY_CUDA(h, cudaGetLastError());
  const double one = 1.0, zero = 0.0;
  if (cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH) != CUBLAS_STATUS_SUCCESS ||
      cublasDgemm(h->cublas, CUBLAS_OP_T, CUBLAS_OP_N, nvec, 3, N, &one, d_A, N, d_D, N, &zero, d_o, nvec) != CUBLAS_STATUS_SUCCESS) {
    h->err = "cx_field_projections: cublasDgemm failed";
    return CX_ERR_LIB;
  }
  CX_TRY_CUDA(h, cudaMemcpyAsync(out, d_o, n_o * 8, cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  return CX_OK;
}
