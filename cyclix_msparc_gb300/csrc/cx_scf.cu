// Self-consistent field loop on the GPU (src/scf.m:1-327, first relaxation step, nspin = 1,
// potential mixing -- the reference defaults of src/initialization.m:1004-1040):
//   Veff0 = phi[rho0] + Vxc[rho0];  loop: eigSolver step; occupations (Fermi level of
//   src/occupations.m); from count >= rhoTrigger: density (src/electronDensity.m:9-12), Poisson
//   (src/poissonSolve.m), Vxc of S.xc: LDA_PW (src/exchangeCorrelationPotential.m:82-106), LDA_PZ
//   or GGA_PBE (:156-362, on the FD gradients of the Cyclix grid), total energy
//   (src/evaluateTotalEnergy.m:12-93) with the Escc correction (src/scf.m:152), error
//   ||Veff - Veff_in|| / ||Veff|| (src/scf.m:177) and Periodic-Pulay mixing (src/mixing.m:20-116).
// All N-length arithmetic is FP64 on the device; the host only drives the loop and reads scalars.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cx_common.h"
#include "cx_xc_point.h"

namespace cx {

constexpr double kXcRhoTol = xc::kRhoTol;   // src/initialization.m:143
static_assert(xc::kGradMaxFDn == kMaxFDn, "gradient stencils cover every supported FD order");
constexpr int kMixHist = 7;           // src/initialization.m:1035

// Fermi level by bisection on sum_b occfac w_b sum_i occ(lambda_i) + NegCharge = 0, then the
// occupations, Eband and Eent (src/occupations.m:1-35, src/evaluateTotalEnergy.m:13-20, 76-90).
// One CTA.  out: [0] lambda_f, [1] Eband, [2] Eent.
__global__ void k_occupations(const double* __restrict__ ev, const double* __restrict__ w_state, int n, double bet, double occfac,
                              double negcharge, int fermi_dirac, double* __restrict__ occ, double* __restrict__ out) {
  __shared__ double red[32];
  __shared__ double lohi[2];
  auto block_sum = [&](double v) -> double {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0) {
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
      red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
  };
  auto occ_of = [&](double lam, double mu) -> double {
    return fermi_dirac ? 1.0 / (1.0 + exp(bet * (lam - mu))) : 0.5 * (1.0 - erf(bet * (lam - mu)));
  };
  double mn = 1e300, mx = -1e300;
  for (int i = threadIdx.x; i < n; i += blockDim.x) { mn = fmin(mn, ev[i]); mx = fmax(mx, ev[i]); }
  for (int o = 16; o > 0; o >>= 1) { mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o)); mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o)); }
  __shared__ double smn[32], smx[32];
  if ((threadIdx.x & 31) == 0) { smn[threadIdx.x >> 5] = mn; smx[threadIdx.x >> 5] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { smn[0] = fmin(smn[0], smn[k]); smx[0] = fmax(smx[0], smx[k]); }
    lohi[0] = smn[0] - 10.0;
    lohi[1] = smx[0] + 10.0;
  }
  __syncthreads();
  for (int it = 0; it < 200; ++it) {
    const double lo = lohi[0], hi = lohi[1];
    const double mid = 0.5 * (lo + hi);
    if (!(hi - lo > 2e-16 * fmax(1.0, fabs(mid)))) break;
    double f = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) f += occfac * w_state[i] * occ_of(ev[i], mid);
    f = block_sum(f) + negcharge;
    if (threadIdx.x == 0) { if (f > 0) lohi[1] = mid; else lohi[0] = mid; }
    __syncthreads();
  }
  const double mu = 0.5 * (lohi[0] + lohi[1]);
  double eb = 0, ee = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double o = occ_of(ev[i], mu);
    occ[i] = o;
    eb += occfac * w_state[i] * ev[i] * o;
    double ent;
    if (fermi_dirac) {
      ent = occfac * (1 / bet) * (o * log(o) + (1 - o) * log(1 - o));
      if (ent != ent) ent = 0.0;
    } else {
      const double x = bet * (ev[i] - mu);
      ent = -occfac * (1 / bet) * 1 / (2 * sqrt(M_PI)) * exp(-x * x);
    }
    ee += w_state[i] * ent;
  }
  eb = block_sum(eb);
  ee = block_sum(ee);
  if (threadIdx.x == 0) { out[0] = mu; out[1] = eb; out[2] = ee; }
}

// rho[p] (+)= fac * sum_j occ_j |psi_j[p]|^2 over the Ns columns of one block (src/electronDensity.m:9-12)
template <typename R>
__global__ void k_density(const cplx<R>* __restrict__ psi, int N, int Ns, const double* __restrict__ occ, double fac, int accumulate,
                          double* __restrict__ rho) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    double acc = 0;
    for (int j = 0; j < Ns; ++j) {
      const cplx<R> v = psi[(size_t)j * N + p];
      acc += occ[j] * ((double)v.x * v.x + (double)v.y * v.y);
    }
    rho[p] = (accumulate ? rho[p] : 0.0) + fac * acc;
  }
}

__global__ void k_poisson_rhs(const double* __restrict__ rho, const double* __restrict__ b, double* __restrict__ f, int N) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) f[p] = -4.0 * M_PI * (rho[p] + b[p]);
}

// block partial sums of kNSums values: one per block in partial[block * kNSums + k]
constexpr int kNSums = 7;
__device__ __forceinline__ void block_partials(const double (&s)[kNSums], double* __restrict__ partial) {
  __shared__ double red[kNSums][32];
#pragma unroll
  for (int k = 0; k < kNSums; ++k) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < kNSums) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
    partial[(size_t)blockIdx.x * kNSums + threadIdx.x] = t;
  }
}

// LDA_PW exchange-correlation (src/exchangeCorrelationPotential.m:82-106 for Vxc,
// src/evaluateTotalEnergy.m:28-43 for the energy density), Veff = phi + Vxc, and the block
// partial sums of: [0] ec rho_c W, [1] rho_c^(4/3) W, [2] Vxc rho_c W, [3] (b - rho) phi W,
// [4] (Veff - Veff_in) rho W, [5] (Veff - Veff_in)^2, [6] Veff^2.
__global__ void k_xc_veff(const double* __restrict__ rho, const double* __restrict__ phi, const double* __restrict__ b,
                          const double* __restrict__ W, const double* __restrict__ veff_in, double* __restrict__ vxc,
                          double* __restrict__ veff, int N, double* __restrict__ partial) {
  double s[kNSums] = {0, 0, 0, 0, 0, 0, 0};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const double r0 = rho[p];
    const double rc = r0 < kXcRhoTol ? kXcRhoTol : r0;
    double v, ec;
    xc::lda_pw(rc, v, ec);
    vxc[p] = v;
    const double ve = phi[p] + v;
    veff[p] = ve;
    const double w = W[p];
    const double d = ve - veff_in[p];
    s[0] += ec * rc * w;
    s[1] += rc * cbrt(rc) * w;
    s[2] += v * rc * w;
    s[3] += (b[p] - r0) * phi[p] * w;
    s[4] += d * r0 * w;
    s[5] += d * d;
    s[6] += ve * ve;
  }
  block_partials(s, partial);
}

// Veff = phi + Vxc for a potential vxc computed before (xc_eval), with the sums of k_xc_veff
// except [0] = rho e_xc W (erho = rho_c e_xc) and [1] = 0, so that Exc = [0] - C2 [1] holds for
// every functional.
__global__ void k_veff_sums(const double* __restrict__ rho, const double* __restrict__ phi, const double* __restrict__ b,
                            const double* __restrict__ W, const double* __restrict__ veff_in, const double* __restrict__ vxc,
                            const double* __restrict__ erho, double* __restrict__ veff, int N, double* __restrict__ partial) {
  double s[kNSums] = {0, 0, 0, 0, 0, 0, 0};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const double r0 = rho[p];
    const double rc = r0 < kXcRhoTol ? kXcRhoTol : r0;
    const double v = vxc[p];
    const double ve = phi[p] + v;
    veff[p] = ve;
    const double w = W[p];
    const double d = ve - veff_in[p];
    s[0] += erho[p] * w;
    s[2] += v * rc * w;
    s[3] += (b[p] - r0) * phi[p] * w;
    s[4] += d * r0 * w;
    s[5] += d * d;
    s[6] += ve * ve;
  }
  block_partials(s, partial);
}

// ---- exchange-correlation potentials on their own (LDA_PW, LDA_PZ, GGA_PBE), for xc_eval
// vxc = d(rho e_xc)/d rho and erho = rho_c e_xc at the clipped density
template <int XC>
__global__ void k_xc_lda(const double* __restrict__ rho, int N, double* __restrict__ vxc, double* __restrict__ erho) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const double r0 = rho[p];
    const double rc = r0 < kXcRhoTol ? kXcRhoTol : r0;
    double v, e;
    if (XC == xc::kLdaPw) {
      xc::lda_pw(rc, v, e);
      e = e * rc - 0.73855876638202 * rc * cbrt(rc);
    } else {
      xc::lda_pz(rc, v, e);
    }
    vxc[p] = v;
    erho[p] = e;
  }
}

// GGA_PBE in two passes over the grid (the per-point arithmetic is xc::gga_pass1_point /
// gga_pass2_point): the flux q of every point must be complete before its divergence is taken.
__global__ void k_gga_pass1(const double* __restrict__ rho, xc::GgaGrid g, int N, double* __restrict__ vxc,
                            double* __restrict__ erho, double* __restrict__ q) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) xc::gga_pass1_point(rho, g, p, vxc, erho, q);
}

__global__ void k_gga_pass2(const double* __restrict__ q, xc::GgaGrid g, int N, double* __restrict__ vxc) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) xc::gga_pass2_point(q, g, p, vxc);
}

// e_xc = erho / rho_c (the energy per particle that exchangeCorrelationPotential stores in S.e_xc)
__global__ void k_exc_per_particle(const double* __restrict__ rho, int N, double* __restrict__ erho) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const double r0 = rho[p];
    erho[p] /= r0 < kXcRhoTol ? kXcRhoTol : r0;
  }
}

__global__ void k_sum_partials(const double* __restrict__ partial, int nblocks, int nsums, double* __restrict__ out) {
  // one warp per sum
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (k >= nsums) return;
  double t = 0;
  for (int i = lane; i < nblocks; i += 32) t += partial[(size_t)i * nsums + k];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[k] = t;
}

// Periodic Pulay (src/mixing.m:29-46): f_k = g_k - x_k and the history columns
__global__ void k_mix_hist(const double* __restrict__ g, const double* __restrict__ x, double* __restrict__ f, double* __restrict__ X,
                           double* __restrict__ F, const double* __restrict__ xkm1, const double* __restrict__ fkm1, int N, int col,
                           int store) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const double fk = g[p] - x[p];
    f[p] = fk;
    if (store) {
      X[(size_t)col * N + p] = x[p] - xkm1[p];
      F[(size_t)col * N + p] = fk - fkm1[p];
    }
  }
}
// normal matrix F'F (m x m) and F'f (m) into io (layout of launch_pinv_solve)
__global__ void k_mix_gram(const double* __restrict__ F, const double* __restrict__ f, int N, int m, double* __restrict__ io) {
  const int i = blockIdx.x / (m + 1), j = blockIdx.x % (m + 1);
  const double* a = F + (size_t)i * N;
  const double* bb = j < m ? F + (size_t)j * N : f;
  double s = 0;
  for (int k = threadIdx.x; k < N; k += blockDim.x) s += a[k] * bb[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    if (j < m) io[i * m + j] = t; else io[m * m + i] = t;
  }
}
// x_{k+1} = x_k - X G + beta (f_k - F G) (Anderson, src/andersonWtdAvg.m:19-21) or x_k + beta f_k;
// then x_{k-1} = x_k, f_{k-1} = f_k
__global__ void k_mix_update(const double* __restrict__ X, const double* __restrict__ F, const double* __restrict__ gamma, int anderson,
                             double beta, double* __restrict__ x, const double* __restrict__ f, double* __restrict__ xkm1,
                             double* __restrict__ fkm1, double* __restrict__ xnew, int N, int m) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    double xw = x[p], fw = f[p];
    if (anderson)
      for (int k = 0; k < m; ++k) {
        xw -= X[(size_t)k * N + p] * gamma[k];
        fw -= F[(size_t)k * N + p] * gamma[k];
      }
    xkm1[p] = x[p];
    fkm1[p] = f[p];
    xnew[p] = xw + beta * fw;
  }
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = (float)a[i];
}

struct ScfBufs {
  double *rho, *b, *phi, *vxc, *vin, *f, *X, *F, *xkm1, *fkm1, *fk, *partial, *sums, *ev, *occ, *wst, *occout, *io;
  double *erho, *q;          // rho e_xc (N) and the GGA flux 2 df/dsigma grad rho (3 N)
  int nred;
};

// State of an SCF run between cx_scf_init and cx_scf_finish (the loop variables of src/scf.m).
struct ScfState {
  cx_scf_params P{};
  ScfBufs B{};
  std::vector<double> wblk, ev, a0, bup, lc, hist;
  double sums[kNSums] = {};
  double ptol = 0, err = 100.0, Etot = 0.0, lam_f = 0.0;
  int pmax = 1000, rhoTrigger = 4, count = 1, count_scf = 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr, p0 = nullptr, p1 = nullptr;
  ~ScfState() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (p0) cudaEventDestroy(p0);
    if (p1) cudaEventDestroy(p1);
  }
};

void scf_state_free(cx_handle h) {
  delete h->scf;
  h->scf = nullptr;
}

template <typename R>
static cx_status density_all(cx_handle h, const ScfBufs& B, const std::vector<double>& wblk) {
  const int N = h->g.N;
  const unsigned gN = (unsigned)std::min(152 * 8, (N + 255) / 256);
  int off = 0;
  for (int b = 0; b < h->nblk; ++b) {
    const cplx<R>* psi = (const cplx<R>*)h->bufs[2 * b + h->psi_sel[0]];
    k_density<R><<<gN, 256, 0, h->stream>>>(psi, N, h->blocks[b].Ns, B.occ + off, 2.0 * wblk[b], b > 0 ? 1 : 0, B.rho);
    h->launches++;
    off += h->blocks[b].Ns;
  }
  CX_TRY_CUDA(h, cudaGetLastError());
  return CX_OK;
}

cx_status eigsolver_dispatch(cx_handle h, int count, int npl, int rhoTrigger, double* EigVal, double* a0, double* bup, double* lc);

static unsigned grid_n(int N) { return (unsigned)std::min(152 * 8, (N + 255) / 256); }

// Vxc and rho e_xc of the functional xc on the device density rho (N each); q: 3 N work values
// for GGA_PBE.  Launches on the handle's stream.
static cx_status xc_eval(cx_handle h, int xc, const double* rho, double* vxc, double* erho, double* q) {
  const int N = h->g.N;
  const unsigned gN = grid_n(N);
  const cudaStream_t st = h->stream;
  if (xc == xc::kLdaPw) {
    k_xc_lda<xc::kLdaPw><<<gN, 256, 0, st>>>(rho, N, vxc, erho);
    h->launches++;
  } else if (xc == xc::kLdaPz) {
    k_xc_lda<xc::kLdaPz><<<gN, 256, 0, st>>>(rho, N, vxc, erho);
    h->launches++;
  } else {
    xc::GgaGrid g{};
    g.Nx = h->g.Nx; g.Ny = h->g.Ny; g.Nz = h->g.Nz; g.FDn = h->g.FDn;
    g.xin = h->grid.xin; g.dx = h->grid.dx; g.dy = h->grid.dy; g.dz = h->grid.dz; g.twist = h->grid.twist;
    for (int k = 1; k <= h->g.FDn; ++k) {
      g.gr[k] = h->w1[k] / h->grid.dx;
      g.gt[k] = h->w1[k] / h->grid.dy;
      g.gz[k] = h->w1[k] / h->grid.dz;
    }
    k_gga_pass1<<<gN, 256, 0, st>>>(rho, g, N, vxc, erho, q);
    k_gga_pass2<<<gN, 256, 0, st>>>(q, g, N, vxc);
    h->launches += 2;
  }
  CX_TRY_CUDA(h, cudaGetLastError());
  return CX_OK;
}

// the functionals cx_scf and cx_xc accept on the handle's grid
static bool xc_supported(cx_handle h, int xc) {
  if (xc == xc::kLdaPw || xc == xc::kLdaPz) return true;
  if (xc != xc::kGgaPbe) {
    h->err = "exchange-correlation code " + std::to_string(xc) + ": 0 LDA_PW, 1 LDA_PZ or 2 GGA_PBE";
    return false;
  }
  if (h->grid.BCy != 0 || h->grid.BCz != 0) {
    h->err = "GGA_PBE: the gradient stencils need periodic theta and z (BCy = BCz = 0)";
    return false;
  }
  return true;
}

// phi = Poisson(rho), Vxc(rho), Veff = phi + Vxc (into h->d_veff) and the energy / error sums
static cx_status scf_potential(cx_handle h, ScfState& S, int use_guess, int* iters, float* pms) {
  const int N = h->g.N;
  const unsigned gN = grid_n(N);
  const cudaStream_t st = h->stream;
  ScfBufs& B = S.B;
  k_poisson_rhs<<<gN, 256, 0, st>>>(B.rho, B.b, B.f, N);
  h->launches++;
  int it = 0;
  double rr = 0;
  CX_TRY_CUDA(h, cudaEventRecord(S.p0, st));
  cx_status s = poisson_dev(h, B.f, B.phi, S.ptol, S.pmax, use_guess, &it, &rr);
  if (s != CX_OK && s != CX_ERR_NOCONV) return s;
  CX_TRY_CUDA(h, cudaEventRecord(S.p1, st));
  if (S.P.xc == xc::kLdaPw) {
    k_xc_veff<<<gN, 256, 0, st>>>(B.rho, B.phi, B.b, h->d_W, B.vin, B.vxc, h->d_veff, N, B.partial);
  } else {
    cx_status xs = xc_eval(h, S.P.xc, B.rho, B.vxc, B.erho, B.q);
    if (xs != CX_OK) return xs;
    k_veff_sums<<<gN, 256, 0, st>>>(B.rho, B.phi, B.b, h->d_W, B.vin, B.vxc, B.erho, h->d_veff, N, B.partial);
  }
  k_sum_partials<<<1, 32 * kNSums, 0, st>>>(B.partial, (int)gN, kNSums, B.sums);
  h->launches += 2;
  CX_TRY_CUDA(h, cudaMemcpyAsync(S.sums, B.sums, sizeof(S.sums), cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  if (iters) *iters = it;
  if (pms) CX_TRY_CUDA(h, cudaEventElapsedTime(pms, S.p0, S.p1));
  return CX_OK;
}

// the block operators read d_veff (complex128 path) and its float copy (complex64 path)
static cx_status scf_refresh_veff(cx_handle h) {
  if (h->d_veff32) {
    k_to_float<<<grid_n(h->g.N), 256, 0, h->stream>>>(h->d_veff, h->d_veff32, h->g.N);
    h->launches++;
  }
  CX_TRY_CUDA(h, cudaGetLastError());
  return CX_OK;
}

static constexpr double kC2 = 0.73855876638202;

static double total_energy(const ScfState& S, const double occout[3]) {
  const double Exc = S.sums[0] - kC2 * S.sums[1], Exc_dc = S.sums[2], Eelec_dc = 0.5 * S.sums[3], Escc = S.sums[4];
  return occout[1] + Exc - Exc_dc + Eelec_dc - S.P.Eself + S.P.E_corr + occout[2] + Escc;
}

}  // namespace cx

using namespace cx;

extern "C" cx_status cx_scf_init(cx_handle h, const cx_scf_params* P) {
  if (!h) return CX_ERR_ARG;
  if (!P) { h->err = "cx_scf_init: null parameters"; return CX_ERR_ARG; }
  if (h->nblk < 1) { h->err = "cx_scf: call cx_set_blocks (and cx_set_psi) first"; return CX_ERR_STATE; }
  if (h->nspin != 1) { h->err = "cx_scf: the SCF driver supports nspin = 1 (spin blocks are supported by cx_eigsolver)"; return CX_ERR_ARG; }
  if (!xc_supported(h, P ? P->xc : 0)) { h->err = "cx_scf: " + h->err; return CX_ERR_ARG; }
  if (!P->b || !P->rho0 || !P->wkpt || P->max_scf < 1 || P->npl < 1 || !(P->scf_tol > 0) || !(P->bet > 0)) {
    h->err = "cx_scf: need b, rho0, wkpt, max_scf >= 1, npl >= 1, scf_tol > 0, bet > 0";
    return CX_ERR_ARG;
  }
  scf_state_free(h);
  ScfState* S = new ScfState();
  h->scf = S;
  S->P = *P;
  S->P.b = S->P.rho0 = nullptr;              // read here only
  const int N = h->g.N, nblk = h->nblk, m = kMixHist;
  const cudaStream_t st = h->stream;
  const unsigned gN = grid_n(N);
  const int ntot = h->nstates;
  CX_TRY_CUDA(h, cudaEventCreate(&S->e0));
  CX_TRY_CUDA(h, cudaEventCreate(&S->e1));
  CX_TRY_CUDA(h, cudaEventCreate(&S->p0));
  CX_TRY_CUDA(h, cudaEventCreate(&S->p1));
  // ---- device buffers
  ScfBufs& B = S->B;
  B.nred = (int)gN;
  const size_t need = (size_t)N * 8 * (13 + 2 * m) + (size_t)gN * kNSums * 8 + 64 * 8 + (size_t)ntot * 8 * 3 + 8 * (m * m + 2 * m + 8) +
                      64 * 256;
  if (h->scf_bytes < need) {
    cudaFree(h->d_scf);
    h->d_scf = nullptr;
    h->scf_bytes = 0;
    CX_TRY_CUDA(h, cudaMalloc(&h->d_scf, need));
    h->scf_bytes = need;
  }
  {
    char* q = (char*)h->d_scf;
    auto take = [&](size_t bytes) { double* o = (double*)q; q += (bytes + 255) & ~(size_t)255; return o; };
    B.rho = take((size_t)N * 8); B.b = take((size_t)N * 8); B.phi = take((size_t)N * 8); B.vxc = take((size_t)N * 8);
    B.vin = take((size_t)N * 8); B.f = take((size_t)N * 8); B.xkm1 = take((size_t)N * 8); B.fkm1 = take((size_t)N * 8);
    B.fk = take((size_t)N * 8); B.X = take((size_t)N * 8 * m); B.F = take((size_t)N * 8 * m);
    B.partial = take((size_t)gN * kNSums * 8); B.sums = take(64 * 8); B.ev = take((size_t)ntot * 8); B.occ = take((size_t)ntot * 8);
    B.wst = take((size_t)ntot * 8); B.occout = take(8 * 8); B.io = take(8 * (m * m + 2 * m + 8));
    B.erho = take((size_t)N * 8); B.q = take((size_t)N * 8 * 3);
  }
  S->wblk.assign(P->wkpt, P->wkpt + nblk);
  std::vector<double> wst(ntot);
  for (int b = 0, o = 0; b < nblk; ++b)
    for (int j = 0; j < h->blocks[b].Ns; ++j) wst[o++] = S->wblk[b];
  CX_TRY_CUDA(h, cudaMemcpyAsync(B.wst, wst.data(), ntot * 8, cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(B.b, P->b, (size_t)N * 8, cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemcpyAsync(B.rho, P->rho0, (size_t)N * 8, cudaMemcpyHostToDevice, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(B.X, 0, (size_t)N * 8 * m, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(B.F, 0, (size_t)N * 8 * m, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(B.fkm1, 0, (size_t)N * 8, st));
  CX_TRY_CUDA(h, cudaMemsetAsync(B.vin, 0, (size_t)N * 8, st));
  S->ptol = P->poisson_tol > 0 ? P->poisson_tol : 0.01 * P->scf_tol;
  S->pmax = P->maxit_poisson > 0 ? P->maxit_poisson : 1000;
  S->rhoTrigger = P->rhoTrigger > 0 ? P->rhoTrigger : 4;
  S->a0.assign(nblk, 0.0);
  S->bup.assign(nblk, 0.0);
  S->lc.assign(nblk, 0.0);
  S->ev.assign(ntot, 0.0);
  S->hist.clear();
  S->count = 1;
  S->count_scf = 1;
  S->err = 100.0;
  S->Etot = S->lam_f = 0.0;
  cx_status s;
  // ---- initial potential (src/scf.m:32-39)
  if ((s = scf_potential(h, *S, 0, nullptr, nullptr)) != CX_OK) return s;
  if ((s = scf_refresh_veff(h)) != CX_OK) return s;
  CX_TRY_CUDA(h, cudaMemcpyAsync(B.vin, h->d_veff, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));   // Veff_temp
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  return CX_OK;
}

extern "C" cx_status cx_scf_step(cx_handle h, double* psi_host, double* EigVal, cx_scf_step_info* info) {
  if (!h) return CX_ERR_ARG;
  if (!h->scf) { h->err = "cx_scf_step: call cx_scf_init first"; return CX_ERR_STATE; }
  ScfState& S = *h->scf;
  ScfBufs& B = S.B;
  const int N = h->g.N, m = kMixHist, ntot = h->nstates;
  const unsigned gN = grid_n(N);
  const cudaStream_t st = h->stream;
  const cx_scf_params& P = S.P;
  cx_status s;
  cx_scf_step_info out{};
  // the caller's psi (S.psi on the host): copied in before the step and out after it
  if (psi_host) {
    size_t off = 0;
    for (int b = 0; b < h->nblk; ++b) {
      if ((s = cx_set_psi(h, b, psi_host + 2 * off)) != CX_OK) return s;
      off += (size_t)N * h->blocks[b].Ns;
    }
  }
  CX_TRY_CUDA(h, cudaEventRecord(S.e0, st));
  if ((s = eigsolver_dispatch(h, S.count, P.npl, S.rhoTrigger, S.ev.data(), S.a0.data(), S.bup.data(), S.lc.data())) != CX_OK) return s;
  CX_TRY_CUDA(h, cudaMemcpyAsync(B.ev, S.ev.data(), ntot * 8, cudaMemcpyHostToDevice, st));
  k_occupations<<<1, 1024, 0, st>>>(B.ev, B.wst, ntot, P.bet, P.occfac, P.NegCharge, P.elec_T_type == 0, B.occ, B.occout);
  h->launches++;
  double occout[3];
  CX_TRY_CUDA(h, cudaMemcpyAsync(occout, B.occout, sizeof(occout), cudaMemcpyDeviceToHost, st));
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  S.lam_f = occout[0];
  if (S.count >= S.rhoTrigger) {
    s = h->prec == CX_PREC_FP64 ? density_all<double>(h, B, S.wblk) : density_all<float>(h, B, S.wblk);
    if (s != CX_OK) return s;
    float pms = 0;
    if ((s = scf_potential(h, S, 1, &out.poisson_iters, &pms)) != CX_OK) return s;
    out.poisson_ms = pms;
    S.Etot = total_energy(S, occout);
    S.err = std::sqrt(S.sums[5]) / std::sqrt(S.sums[6]);
    S.hist.push_back(S.Etot / std::max(1, P.n_atm));
    S.hist.push_back(S.err);
    if (S.err > P.scf_tol || S.count_scf < P.min_scf) {
      // potential mixing of the mean-free Veff (the mean is 0 for non-periodic cells, src/scf.m:201-215)
      const int col = (S.count_scf - 2 + m) % m;
      k_mix_hist<<<gN, 256, 0, st>>>(h->d_veff, B.vin, B.fk, B.X, B.F, B.xkm1, B.fkm1, N, col, S.count_scf > 1 ? 1 : 0);
      h->launches++;
      const int anderson = S.count_scf > 1 ? 1 : 0;     // PulayFrequency = 1
      if (anderson) {
        k_mix_gram<<<m * (m + 1), 256, 0, st>>>(B.F, B.fk, N, m, B.io);
        CX_TRY_CUDA(h, launch_pinv_solve(B.io, m, st));
        h->launches += 2;
      }
      k_mix_update<<<gN, 256, 0, st>>>(B.X, B.F, B.io + m * m + m, anderson, P.mixing_param > 0 ? P.mixing_param : 0.3, B.vin, B.fk,
                                       B.xkm1, B.fkm1, h->d_veff, N, m);
      h->launches++;
      CX_TRY_CUDA(h, cudaMemcpyAsync(B.vin, h->d_veff, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
    }
    if ((s = scf_refresh_veff(h)) != CX_OK) return s;
    S.count_scf++;
    out.density_updated = 1;
  }
  S.count++;
  CX_TRY_CUDA(h, cudaEventRecord(S.e1, st));
  CX_TRY_CUDA(h, cudaEventSynchronize(S.e1));
  float ms = 0;
  CX_TRY_CUDA(h, cudaEventElapsedTime(&ms, S.e0, S.e1));
  if (psi_host) {
    size_t off = 0;
    for (int b = 0; b < h->nblk; ++b) {
      if ((s = cx_get_psi(h, b, psi_host + 2 * off)) != CX_OK) return s;
      off += (size_t)N * h->blocks[b].Ns;
    }
  }
  if (EigVal) std::copy(S.ev.begin(), S.ev.end(), EigVal);
  out.step_ms = ms;
  out.filter_ms = h->last_filter_ms;
  out.rr_ms = h->last_rr_ms;
  out.Etotal = S.Etot;
  out.lambda_f = S.lam_f;
  out.err = S.err;
  out.count = S.count - 1;
  out.n_scf = S.count_scf - 1;
  out.converged = (S.count_scf - 1 >= 1 && S.err <= P.scf_tol && S.count_scf > P.min_scf) ? 1 : 0;
  if (info) *info = out;
  return CX_OK;
}

extern "C" cx_status cx_scf_finish(cx_handle h, double* EigVal, double* rho_out, double* Veff_out, cx_scf_result* res) {
  if (!h) return CX_ERR_ARG;
  if (!h->scf) { h->err = "cx_scf_finish: call cx_scf_init first"; return CX_ERR_STATE; }
  ScfState& S = *h->scf;
  ScfBufs& B = S.B;
  const int N = h->g.N, ntot = h->nstates;
  const cudaStream_t st = h->stream;
  const cx_scf_params& P = S.P;
  CX_TRY_CUDA(h, cudaStreamSynchronize(st));
  if (P.refine && S.count_scf > 1) {
    // final FP64 refinement step: Rayleigh quotients of the psi of the last step under the potential
    // they were computed for (Veff_in), then occupations, band and entropy energy again; the
    // density-dependent terms of the last step are kept (the energy is stationary in them)
    CX_TRY_CUDA(h, cudaMemcpyAsync(B.f, h->d_veff, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
    CX_TRY_CUDA(h, cudaMemcpyAsync(h->d_veff, B.vin, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
    cx_status s = refine_eigenvalues(h, S.ev.data());
    CX_TRY_CUDA(h, cudaMemcpyAsync(h->d_veff, B.f, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
    if (s != CX_OK) return s;
    CX_TRY_CUDA(h, cudaMemcpyAsync(B.ev, S.ev.data(), ntot * 8, cudaMemcpyHostToDevice, st));
    k_occupations<<<1, 1024, 0, st>>>(B.ev, B.wst, ntot, P.bet, P.occfac, P.NegCharge, P.elec_T_type == 0, B.occ, B.occout);
    h->launches++;
    double occout[3];
    CX_TRY_CUDA(h, cudaMemcpyAsync(occout, B.occout, sizeof(occout), cudaMemcpyDeviceToHost, st));
    CX_TRY_CUDA(h, cudaStreamSynchronize(st));
    S.Etot = total_energy(S, occout);
    S.lam_f = occout[0];
  }
  if (EigVal) std::copy(S.ev.begin(), S.ev.end(), EigVal);
  if (rho_out) CX_TRY_CUDA(h, cudaMemcpy(rho_out, B.rho, (size_t)N * 8, cudaMemcpyDeviceToHost));
  if (Veff_out) CX_TRY_CUDA(h, cudaMemcpy(Veff_out, h->d_veff, (size_t)N * 8, cudaMemcpyDeviceToHost));
  if (res) {
    res->Etotal = S.Etot;
    res->lambda_f = S.lam_f;
    res->err = S.err;
    res->n_scf = S.count_scf - 1;
    res->converged = S.err <= P.scf_tol ? 1 : 0;
  }
  return CX_OK;
}

extern "C" cx_status cx_scf(cx_handle h, const cx_scf_params* P, double* EigVal, double* rho_out, double* Veff_out, double* hist,
                            cx_scf_result* res) {
  if (!h || !P || !EigVal || !res) return CX_ERR_ARG;
  cx_status s = cx_scf_init(h, P);
  if (s != CX_OK) return s;
  ScfState& S = *h->scf;
  // src/scf.m:111: while (err > tol && count_SCF <= MAXIT_SCF) || count_SCF <= MINIT_SCF
  while ((S.err > P->scf_tol && S.count_scf <= P->max_scf) || S.count_scf <= P->min_scf) {
    if ((s = cx_scf_step(h, nullptr, nullptr, nullptr)) != CX_OK) return s;
    if (S.count > 10 * (P->max_scf + S.rhoTrigger)) break;
  }
  if (P->fp64_tol > 0 && h->prec == CX_PREC_MIXED) {
    // FP64 finish: the same blocks in complex128 with the converted psi; the SCF state (potential,
    // density, mixing history, bounds) carries over
    const std::vector<cx_block> blocks = h->blocks;
    std::vector<std::vector<double>> psi(blocks.size());
    for (size_t b = 0; b < blocks.size(); ++b) {
      psi[b].resize((size_t)2 * h->g.N * blocks[b].Ns);
      if ((s = cx_get_psi(h, (int)b, psi[b].data())) != CX_OK) return s;
    }
    if ((s = cx_set_blocks(h, (int)blocks.size(), blocks.data(), CX_PREC_FP64)) != CX_OK) return s;
    for (size_t b = 0; b < blocks.size(); ++b)
      if ((s = cx_set_psi(h, (int)b, psi[b].data())) != CX_OK) return s;
    // the passes mix until the FP64 tolerance is met (the step mixes while err > its scf_tol)
    S.P.scf_tol = P->fp64_tol;
    const int start = S.count_scf;
    while (S.err > P->fp64_tol && S.count_scf - start < P->max_scf) {
      if ((s = cx_scf_step(h, nullptr, nullptr, nullptr)) != CX_OK) return s;
      if (S.count > 10 * (2 * P->max_scf + S.rhoTrigger)) break;
    }
  }
  if (hist) {
    const size_t cap = (P->fp64_tol > 0 ? 4 : 2) * (size_t)P->max_scf;   // rows: max_scf, or 2 max_scf with the FP64 finish
    for (size_t i = 0; i < S.hist.size() && i < cap; ++i) hist[i] = S.hist[i];
  }
  return cx_scf_finish(h, EigVal, rho_out, Veff_out, res);
}

extern "C" cx_status cx_xc(cx_handle h, int32_t xc, const double* rho, double* Vxc, double* e_xc) {
  if (!h) return CX_ERR_ARG;
  if (!rho || !Vxc || !e_xc) { h->err = "cx_xc: rho, Vxc and e_xc are required"; return CX_ERR_ARG; }
  if (!xc_supported(h, xc)) { h->err = "cx_xc: " + h->err; return CX_ERR_ARG; }
  const int N = h->g.N;
  const cudaStream_t st = h->stream;
  double* d = nullptr;                       // rho, Vxc, rho e_xc, 3 N GGA work values
  if (cudaMalloc(&d, (size_t)N * 8 * 6) != cudaSuccess) {
    cudaGetLastError();
    h->err = "cx_xc: device allocation failed";
    return CX_ERR_NOMEM;
  }
  double *d_rho = d, *d_vxc = d + N, *d_e = d + 2 * (size_t)N, *d_q = d + 3 * (size_t)N;
  cx_status s = CX_OK;
  cudaError_t e = cudaMemcpyAsync(d_rho, rho, (size_t)N * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) s = xc_eval(h, xc, d_rho, d_vxc, d_e, d_q);
  if (e == cudaSuccess && s == CX_OK) {
    k_exc_per_particle<<<grid_n(N), 256, 0, st>>>(d_rho, N, d_e);
    h->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && s == CX_OK) e = cudaMemcpyAsync(Vxc, d_vxc, (size_t)N * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && s == CX_OK) e = cudaMemcpyAsync(e_xc, d_e, (size_t)N * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  if (e != cudaSuccess) {
    h->err = std::string("cx_xc: ") + cudaGetErrorString(e);
    return CX_ERR_CUDA;
  }
  return s;
}
