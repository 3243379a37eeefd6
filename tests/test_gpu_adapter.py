"""The C++ façade (foamadapter_gb300/adapter/fvgb_neon.hpp) used the way a
FoamAdapter solver would use NeoN: a compiled C++ heat-transfer program that
steps through the solver options of a mapped fvSolution entry (Jacobi, ILU(0),
BiCG, the ||b|| baseline, the multigrid solver), its results compared with the
CPU oracle running the same steps: bit for bit, the multigrid step to 1e-9."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from foamadapter_gb300 import abi, mesh
from oracle.pyoracle import Oracle

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "heat_adapter.cpp"
OUT = ROOT / "tests" / "cpp" / "_build"


def build_program() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    exe = OUT / "heat_adapter"
    lib = ROOT / "foamadapter_gb300" / "_lib"
    cmd = ["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{ROOT / 'foamadapter_gb300' / 'adapter'}",
           "-I/usr/local/cuda/include", str(SRC), "-o", str(exe), f"-L{lib}", "-lfvgb",
           "-L/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{lib}", "-Wl,-rpath,/usr/local/cuda/lib64"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_program_compiles():
    """The façade header compiles and links against libfvgb (no GPU needed)."""
    assert build_program().exists()


@pytest.mark.gpu
def test_adapter_heat_transfer_matches_oracle(cuda, tmp_path):
    exe = build_program()
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    hm = mesh.box(20, 16, 12, 1.0, 0.8, 0.6, jitter=0.1, seed=12345)
    data = np.fromfile(out, dtype=np.float64)
    n = hm.n
    T1, T2, T3, T4, div_gpu, grad_gpu, T5 = np.split(data, [n, 2 * n, 3 * n, 4 * n, 5 * n, 8 * n])
    o = Oracle(hm)
    k = 1.0 + 0.5 * np.sin(0.37 * np.arange(hm.n))
    kf = o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
    types = np.asarray([abi.BC_FIXED_VALUE] + [abi.BC_FIXED_GRADIENT] * (hm.npatch - 1), np.int32)
    ref = np.zeros(hm.nbf)
    ref[hm.patch_slice("xmin")] = 400.0
    T = np.full(hm.n, 300.0)
    Tb = np.zeros(hm.nbf)
    o.bc_correct(1, types, ref, T, Tb)
    def step(**kw):
        v, rhs, _, _ = o.assemble(1, [(abi.TERM_DDT, 0, 1.0, T.copy(), None),
                                      (abi.TERM_LAPLACIAN, 0, -1.0, None, kf)], 0.01, types, ref, Tb)
        st = o.solve(v, rhs, T, **kw)
        assert st.status == 0
        o.bc_correct(1, types, ref, T, Tb)
        return v, rhs

    for _ in range(3):
        step(rel_tol=1e-8)
    np.testing.assert_array_equal(T1, T)                # CG + Jacobi
    for _ in range(2):
        step(rel_tol=1e-8, preconditioner=2)
    np.testing.assert_array_equal(T2, T)                # CG + ILU(0)
    step(rel_tol=1e-8, method=2)
    np.testing.assert_array_equal(T3, T)                # BiCG
    step(rel_tol=1e-6, flags=2)
    np.testing.assert_array_equal(T4, T)                # ||r|| <= 1e-6 ||b||
    U = np.tile([1.0, 0.5, 0.25], hm.n)
    Ub = np.tile([1.0, 0.5, 0.25], hm.nbf)
    F = o.flux_vec(U, Ub)
    np.testing.assert_array_equal(div_gpu, o.div(abi.SCHEME_UPWIND, 1, F, T, Tb, 1.0, np.zeros(hm.n)))
    np.testing.assert_array_equal(grad_gpu, o.grad(T, Tb, 1.0, np.zeros(3 * hm.n)))
    # the multigrid solver: against the numpy restatement, to its rounding
    from oracle import amg as oamg
    v, rhs, _, _ = o.assemble(1, [(abi.TERM_DDT, 0, 1.0, T.copy(), None),
                                  (abi.TERM_LAPLACIAN, 0, -1.0, None, kf)], 0.01, types, ref, Tb)
    ro, col = o.csr_arrays()[:2]
    x, it, _, _, status = oamg.mg_solve(oamg.hierarchy(ro, col, v), rhs, T.copy(), 1e-8, 0.0, 1000)
    assert status == 0 and it > 2
    assert np.linalg.norm(T5 - x) <= 1e-9 * np.linalg.norm(x)
