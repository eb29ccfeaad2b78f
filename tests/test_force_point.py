"""The nonlocal-force and gradient arithmetic of the GPU kernels, compiled for the host, against the oracle.

``cyclix_msparc_gb300/csrc/cx_force_point.h`` holds the per-point code of cx_force.cu: the segment
table (Bloch phase and wedge / helical rotation of every atom image), the three Bloch-summed
projector fields, their W-weighted Cartesian gradients (the x / y pair rotated across the theta
wrap), the force accumulation from psi^H [W Ck | W D Ck], and the k = 0 gradient of a real field.
Compiled by g++ and driven here with the projector tables cx_create builds (per-point entries of
(segment, chi)), it must reproduce oracle/forces.py (src/atomicForce.m:254-300,
Cychel/div_gradvec_cychel.m, Cychel/blochGradient_cychel.m) on helical and cyclic cells at
Bloch vectors with nonzero theta and z components.  Tolerances: fields 1e-12 relative to the
largest value, forces 1e-10 relative to the largest component."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, initial_psi, make_system

ROOT = Path(__file__).resolve().parents[1]

SHIM = r"""
#include "cx_force_point.h"
using namespace cx::force;
extern "C" {
static ForceGrid grid(const int* dims, const double* geo, const double* w1) {
  ForceGrid g{};
  g.Nx = dims[0]; g.Ny = dims[1]; g.Nz = dims[2]; g.FDn = dims[3];
  g.xin = geo[0]; g.dx = geo[1]; g.dy = geo[2]; g.dz = geo[3]; g.twist = geo[4];
  g.cL2 = cos(geo[5]); g.sL2 = sin(geo[5]);
  for (int q = 0; q <= g.FDn; ++q) g.w1[q] = w1[q];
  return g;
}
// geo: xin dx dy dz twist L2 L3
void fields_grad(const int* dims, const double* geo, const double* w1, const double* k, int C, const int* row_ptr,
                 const int* ent_seg, const double* ent_chi, int nseg, const int* seg_atom, const double* seg_coord,
                 const double* atom_pos, const double* W, double* out) {
  ForceGrid g = grid(dims, geo, w1);
  set_bloch_phases(g, k, geo[5], geo[6]);
  SegForce* seg = new SegForce[nseg];
  segment_table(nseg, seg_atom, seg_coord, atom_pos, k, geo[5], geo[6], geo[4], seg);
  const size_t N = (size_t)g.Nx * g.Ny * g.Nz;
  Cd* f = new Cd[3 * N * C];
  for (size_t p = 0; p < N; ++p) force_fields_point((int)p, N, C, row_ptr, ent_seg, ent_chi, seg, f, f + N * C, f + 2 * N * C);
  for (int c = 0; c < C; ++c)
    for (size_t p = 0; p < N; ++p) force_grad_point((int)p, N, C, c, g, f, f + N * C, f + 2 * N * C, W, (Cd*)out);
  delete[] f;
  delete[] seg;
}
void accumulate(int Ns, int nat, const double* P, const double* occ, const double* gamma, double scale, double* F) {
  force_accumulate(Ns, nat, (const Cd*)P, occ, gamma, scale, F);
}
void real_grad(const int* dims, const double* geo, const double* w1, const double* u, double* D) {
  ForceGrid g = grid(dims, geo, w1);
  const int N = g.Nx * g.Ny * g.Nz;
  for (int p = 0; p < N; ++p) real_grad_point(p, g, u, D);
}
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("force")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "shim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(ROOT / "cyclix_msparc_gb300" / "csrc"),
                    str(d / "shim.cpp"), "-o", str(so)], check=True, capture_output=True, text=True)
    return C.CDLL(str(so))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def projector_tables(S):
    """The tables cx_create builds from S.Atom (4 columns per atom): per-point CSR of
    (segment, chi) entries, segment -> atom, image coordinates, atom positions, gamma."""
    N = S.N
    seg_atom, seg_coord, ents = [], [], [[] for _ in range(N)]
    for J, A in enumerate(S.Atom):
        assert A.angnum <= 4
        for img in A.rcImage:
            s = len(seg_atom)
            seg_atom.append(J)
            seg_coord.append(np.asarray(img.coordinates, float))
            for n, pos in enumerate(np.asarray(img.rc_pos) - 1):
                chi = np.zeros(4)
                chi[:A.angnum] = img.Chi_mat[n, :A.angnum]
                ents[pos].append((s, chi))
    row_ptr = np.zeros(N + 1, np.int32)
    row_ptr[1:] = np.cumsum([len(e) for e in ents])
    ent_seg = np.array([s for e in ents for (s, _) in e], np.int32)
    ent_chi = np.array([c for e in ents for (_, c) in e]).reshape(-1)
    gamma = np.zeros((len(S.Atom), 4))
    for J, A in enumerate(S.Atom):
        gamma[J, :A.angnum] = A.gamma_Jl
    return dict(row_ptr=row_ptr, ent_seg=ent_seg, ent_chi=np.ascontiguousarray(ent_chi), seg_atom=np.array(seg_atom, np.int32),
                seg_coord=np.ascontiguousarray(np.array(seg_coord).reshape(-1)),
                atom_pos=np.ascontiguousarray(np.asarray(S.Atoms, float).reshape(-1)), gamma=np.ascontiguousarray(gamma.reshape(-1)))


def _grid(S):
    dims = np.array([S.Nx, S.Ny, S.Nz, S.FDn], np.int32)
    geo = np.array([S.xin, S.dx, S.dy, S.dz, S.twist, S.L2, S.L3])
    return dims, geo, np.ascontiguousarray(S.w1, dtype=np.float64)


CELLS = ["scf-small-helical-24x12x16-8at-2k-ns28", "scf-small-24x12x20-12at-2k-ns40"]


@pytest.fixture(scope="module", params=CELLS, ids=["helical", "cyclic"])
def cell(request):
    wl = WORKLOADS[request.param]
    S = make_system(wl)
    return S, block_layout(wl, S), projector_tables(S)


def _fields(lib, S, T, k):
    dims, geo, w1 = _grid(S)
    nat = len(S.Atom)
    Cc = 4 * nat
    out = np.zeros(2 * 4 * S.N * Cc)
    kk = np.ascontiguousarray(k, dtype=np.float64)
    lib.fields_grad(_p(dims), _p(geo), _p(w1), _p(kk), Cc, _p(T["row_ptr"]), _p(T["ent_seg"]), _p(T["ent_chi"]),
                    len(T["seg_atom"]), _p(T["seg_atom"]), _p(T["seg_coord"]), _p(T["atom_pos"]),
                    _p(np.ascontiguousarray(S.W, dtype=np.float64)), _p(out))
    return out.view(np.complex128).reshape(4, Cc, S.N)          # [W Ck | W Dx | W Dy | W Dz], column c, point


def test_projector_gradient_fields_match_oracle(lib, cell):
    from oracle.forces import projector_gradients
    S, blocks, T = cell
    for k in ([0.0, 1.3, 0.7], list(blocks[-1][0])):
        out = _fields(lib, S, T, k)
        for J, A in enumerate(S.Atom):
            ref = projector_gradients(S, J, np.asarray(k, float))
            for q in range(4):
                R = ref[q] * S.W[:, None]                         # N x angnum
                G = out[q, 4 * J:4 * J + A.angnum].T
                assert np.max(np.abs(G - R)) <= 1e-12 * max(np.max(np.abs(R)), 1e-300), (J, q, k)


def test_nonlocal_force_matches_oracle(lib, cell):
    from oracle.forces import nonlocal_forces
    S, blocks, T = cell
    rng = np.random.default_rng(5)
    nat = len(S.Atom)
    F = np.zeros(3 * nat)
    kv, wk, psis, occs = [], [], [], []
    for b, (k, _, n) in enumerate(blocks):
        psi = initial_psi(S.N, n, 11 + b)
        occ = rng.uniform(0, 1, n)
        w = 0.5 + 0.25 * b
        out = _fields(lib, S, T, k).reshape(4 * 4 * nat, S.N).T        # N x 4C
        P = np.ascontiguousarray((psi.conj().T @ out).T)               # Ns x 4C, column-major
        lib.accumulate(n, nat, _p(P.view(np.float64)), _p(np.ascontiguousarray(occ)), _p(T["gamma"]), C.c_double(2.0 * 2.0 * w), _p(F))
        kv.append(np.asarray(k, float)); wk.append(w); psis.append(psi); occs.append(occ)
    ref = nonlocal_forces(S, kv, wk, psis, occs, 2.0)
    got = F.reshape(3, nat).T
    assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref))


def test_real_gradient_matches_oracle(lib, cell):
    from oracle.forces import bloch_gradients
    S, _, _ = cell
    dims, geo, w1 = _grid(S)
    u = np.random.default_rng(3).standard_normal(S.N)
    D = np.zeros(3 * S.N)
    lib.real_grad(_p(dims), _p(geo), _p(w1), _p(u), _p(D))
    for d, G in enumerate(bloch_gradients(S, (0.0, 0.0, 0.0))):
        ref = (G @ u).real
        assert np.max(np.abs(D[d * S.N:(d + 1) * S.N] - ref)) <= 1e-12 * np.max(np.abs(ref))
