"""OpenFOAM dictionaries and the fvSolution / fvSchemes mapping (host code).

The expected values are those of the reference's own tests on its own case
files: test/test_readDict.cpp:11-91 (convert of testDictionary and of the
setup_operator fvSchemes, which #includes simulationParameters and expands
$GRADSCHEME), test/test_compatibility.cpp:23-86 (updateSolver,
updatePreconditioner), and the mapping rules of
src/compatibility/fvSolution.cpp:19-159.
"""
from __future__ import annotations

import pytest

from conftest import unpack_reference_dicts
from foamadapter_gb300 import abi
from foamadapter_gb300.dictionary import (Dictionary, map_fv_solution, scheme, solver_config, update_criteria,
                                          update_preconditioner, update_solver)


@pytest.fixture(scope="module")
def ref(tmp_path_factory):
    return unpack_reference_dicts(tmp_path_factory.mktemp("dicts"))


def test_every_reference_dictionary_parses(ref):
    files = sorted(p for p in ref.rglob("system/*") if p.is_file())
    assert len(files) >= 60
    for p in files:
        d = Dictionary.read(p)
        assert "FoamFile" not in d.keys(), p


def test_read_test_dictionary(ref):
    # test_readDict.cpp:67-91
    d = Dictionary.read(ref / "test/setup_operator/system/testDictionary")
    assert d.get("label") == 1 and isinstance(d.get("label"), int)
    assert d.get("scalar") == 2.1
    assert d.get("scalar2") == 2.0 and isinstance(d.get("scalar2"), float)
    assert d.get("scalarWriteAnsInt") == 2 and isinstance(d.get("scalarWriteAnsInt"), int)
    assert d.get("vector") == (1.0, 2.0, 3.0)
    assert d.get("word") == "word"
    sub = d.subDict("subDict")
    assert sub.get("subScalar") == 4.1
    assert sub.get("subVector") == (5.0, 6.0, 7.0)
    assert sub.get("subWord") == "subWord"


def test_read_fv_schemes_with_include_and_variables(ref):
    # test_readDict.cpp:40-65
    d = Dictionary.read(ref / "test/setup_operator/system/fvSchemes")
    assert d.subDict("ddtSchemes").get("ddt(T)") == "Euler"
    assert d.subDict("gradSchemes").get("limited") == ["cellLimited", "Gauss", "linear", 1]
    assert d.subDict("gradSchemes").get("grad(U)") == ["Gauss", "linear"]
    assert d.subDict("laplacianSchemes").get("laplacian(Gamma,T)") == ["Gauss", "linear", "uncorrected"]
    # the included file's entries are part of the dictionary, as in OpenFOAM
    assert d.get("NX") == 5


@pytest.mark.parametrize("name,ginkgo", [("PCG", "solver::Cg"), ("PBiCG", "solver::Bicg"),
                                         ("PBiCGStab", "solver::Bicgstab"), ("smoothSolver", "solver::Bicgstab"),
                                         ("GAMG", "solver::Multigrid")])
def test_update_solver(ref, name, ginkgo):
    # test_compatibility.cpp:38-61
    fv = Dictionary.read(ref / "test/setup_compatibility/system/fvSolution")
    s1 = fv.subDict("solvers").subDict("solver1")
    s1.insert("solver", name)
    update_solver(s1)
    assert s1.get("solver") == "Ginkgo"
    assert s1.get("type") == ginkgo


def test_update_solver_leaves_unknown_names():
    d = Dictionary.parse("solver Ginkgo; type \"solver::Cg\";")
    update_solver(d)
    assert d.get("solver") == "Ginkgo" and d.get("type") == "solver::Cg"
    with pytest.raises(abi.FvgbError):
        update_solver(Dictionary.parse("tolerance 1e-6;"))


def test_update_preconditioner(ref):
    # test_compatibility.cpp:63-85
    fv = Dictionary.read(ref / "test/setup_compatibility/system/fvSolution")
    s1 = fv.subDict("solvers").subDict("solver1")
    s1.insert("preconditioner", "DIC")
    update_preconditioner(s1)
    p = s1.subDict("preconditioner")
    assert p.get("type") == "preconditioner::Jacobi"
    assert p.get("max_block_size") == 1
    s1.insert("preconditioner", "DILU")
    update_preconditioner(s1)
    p = s1.subDict("preconditioner")
    assert p.get("type") == "preconditioner::Ilu"
    assert p.get_bool("reverse_apply") is False
    assert p.subDict("factorization").get("type") == "factorization::ParIlu"


def test_update_preconditioner_default_and_smoother():
    # fvSolution.cpp:65-73: no preconditioner -> DIC; a smoother entry is dropped
    d = Dictionary.parse("solver smoothSolver; smoother symGaussSeidel; tolerance 1e-05; relTol 0;")
    update_preconditioner(d)
    assert "smoother" not in d
    assert d.subDict("preconditioner").get("type") == "preconditioner::Jacobi"
    # fvSolution.cpp:75-91: a preconditioner dictionary whose type is itself a dictionary
    gamg = Dictionary.parse("solver PCG; preconditioner { type { name GAMG; } }")
    with pytest.raises(abi.FvgbError) as e:
        update_preconditioner(gamg)
    assert e.value.status == abi.ERR_UNSUPPORTED
    # an unmapped word stays
    d = Dictionary.parse("solver PCG; preconditioner none;")
    update_preconditioner(d)
    assert d.get("preconditioner") == "none"


def test_update_criteria():
    # fvSolution.cpp:106-142
    d = Dictionary.parse("solver PCG; tolerance 1e-8; relTol 1e-5; maxIter 250;")
    update_criteria(d)
    c = d.subDict("criteria")
    assert c.get("iteration") == 250
    assert c.get("relative_residual_norm") == 1e-5
    assert c.get("absolute_residual_norm") == 1e-8
    for k in ("tolerance", "relTol", "maxIter"):
        assert k not in d
    d = Dictionary.parse("solver PCG;")
    update_criteria(d)
    assert d.subDict("criteria").keys() == ["iteration"] and d.subDict("criteria").get("iteration") == 1000


def test_map_cavity_fv_solution(ref):
    # tutorials/cavity: pFinal { $p; relTol 0; }, neoIcoFoam.cpp:38-42 maps p and U
    fv = Dictionary.read(ref / "tutorials/cavity/system/fvSolution")
    solvers = fv.subDict("solvers")
    pf = solvers.subDict("pFinal")
    assert pf.get("solver") == "PCG" and pf.get("preconditioner") == "DIC"
    assert pf.get("tolerance") == 1e-6 and pf.get("relTol") == 0
    p = map_fv_solution(solvers.subDict("p"))
    assert solvers.subDict("p").get("solver") == "PCG"  # mapFvSolution returns a copy
    assert p.get("solver") == "Ginkgo" and p.get("type") == "solver::Cg"
    assert p.subDict("preconditioner").get("type") == "preconditioner::Jacobi"
    assert p.subDict("criteria").get("absolute_residual_norm") == 1e-6
    assert p.subDict("criteria").get("relative_residual_norm") == 0.0
    cfg = solver_config(p)
    assert cfg["method"] == abi.SOLVER_CG and cfg["abs_tol"] == 1e-6 and cfg["rel_tol"] == 0.0
    assert cfg["max_iter"] == 1000 and cfg["precision"] == abi.PREC_FP64
    U = map_fv_solution(solvers.subDict("U"))
    assert U.get("type") == "solver::Bicgstab" and "smoother" not in U
    assert solver_config(U)["method"] == abi.SOLVER_BICGSTAB
    # Ginkgo-form entries go through unchanged
    nfP = solvers.subDict("nfP")
    assert nfP.get("type") == "solver::Cg"
    assert nfP.subDict("criteria").get("relative_residual_norm") == 1e-7


def test_solver_config_rejects_what_is_not_built(ref):
    adv = Dictionary.read(ref / "test/setup_advection/system/fvSolution")
    m = map_fv_solution(adv.subDict("solvers").subDict("T"))  # PBiCGStab + DILU
    assert m.subDict("preconditioner").get("type") == "preconditioner::Ilu"
    c = solver_config(m)  # DILU -> Ilu/ParIlu: the ILU(0) preconditioner around BiCGStab
    assert c["method"] == abi.SOLVER_BICGSTAB and c["preconditioner"] == abi.PRECOND_ILU
    assert c["abs_tol"] == 1e-14 and c["rel_tol"] == 0.0
    with pytest.raises(abi.FvgbError) as e:  # BiCG with ILU is not built
        solver_config(map_fv_solution(Dictionary.parse("solver PBiCG; preconditioner DILU;")))
    assert e.value.status == abi.ERR_UNSUPPORTED
    with pytest.raises(abi.FvgbError) as e:
        solver_config(Dictionary.parse('solver Ginkgo; type "solver::Cg"; preconditioner { type '
                                       '"preconditioner::Ilu"; reverse_apply true; }'))
    assert e.value.status == abi.ERR_UNSUPPORTED
    # GAMG maps to Ginkgo's solver::Multigrid as the solver, which is built; the
    # smoother entry is dropped and the DIC (Jacobi) preconditioner inserted
    gamg = solver_config(map_fv_solution(Dictionary.parse(
        "solver GAMG; smoother GaussSeidel; tolerance 0; relTol 1e-7; maxIter 300;")))
    assert gamg["method"] == abi.SOLVER_MULTIGRID and gamg["rel_tol"] == 1e-7 and gamg["max_iter"] == 300
    with pytest.raises(abi.FvgbError) as e:
        solver_config(map_fv_solution(Dictionary.parse("solver GAMG; preconditioner DILU;")))
    assert e.value.status == abi.ERR_UNSUPPORTED
    # PBiCG maps to Ginkgo's solver::Bicg, which is built
    bicg = solver_config(map_fv_solution(Dictionary.parse("solver PBiCG; preconditioner DIC; relTol 1e-6;")))
    assert bicg["method"] == abi.SOLVER_BICG and bicg["rel_tol"] == 1e-6
    with pytest.raises(abi.FvgbError):
        solver_config(Dictionary.parse("solver PCG;"))  # not mapped
    cfg = Dictionary.parse("configFile \"gko/config.bj.json\";")
    assert map_fv_solution(cfg).keys() == ["configFile"]
    with pytest.raises(ValueError):
        solver_config(cfg)  # a configFile needs the directory it is relative to


def test_solver_config_extensions():
    m = map_fv_solution(Dictionary.parse(
        "solver PCG; preconditioner DIC; tolerance 0; relTol 1e-8; precision mixed; innerRelTol 0.05; maxOuter 7;"))
    cfg = solver_config(m)
    assert cfg["precision"] == abi.PREC_MIXED_IR and cfg["inner_rel_tol"] == 0.05 and cfg["max_outer"] == 7
    assert cfg["rel_tol"] == 1e-8
    m = map_fv_solution(Dictionary.parse("solver PBiCGStab; preconditioner DIC;"))
    assert solver_config(m)["inner_rel_tol"] == 0.01


@pytest.mark.parametrize("case,section,name,want", [
    ("tutorials/scalarAdvection", "divSchemes", "div(phi,T)", abi.SCHEME_UPWIND),
    ("tutorials/scalarAdvection", "gradSchemes", "grad(T)", abi.SCHEME_LINEAR),
    ("tutorials/scalarAdvection", "ddtSchemes", "ddt(T)", 0),
    ("tutorials/heatTranfer3D", "laplacianSchemes", "laplacian(kappa,T)", 0),
    ("tutorials/heatTranfer3D", "interpolationSchemes", "interpolate(T)", abi.SCHEME_LINEAR),
    ("tutorials/heatTranfer3D", "snGradSchemes", "snGrad(T)", 0),
    ("tutorials/heatTranfer3D", "gradSchemes", "grad(T)", abi.SCHEME_LINEAR),
    ("test/setup_operator", "divSchemes", "div(phi,T)", abi.SCHEME_LINEAR),
    ("test/setup_operator", "laplacianSchemes", "laplacian(Gamma,T)", 0),
])
def test_schemes(ref, case, section, name, want):
    fs = Dictionary.read(ref / case / "system/fvSchemes")
    assert scheme(fs, section, name) == want


def test_scheme_errors(ref):
    fs = Dictionary.read(ref / "tutorials/scalarAdvection/system/fvSchemes")
    with pytest.raises(abi.FvgbError) as e:
        scheme(fs, "laplacianSchemes", "laplacian(k,T)")  # default none
    assert e.value.status == abi.ERR_INVALID_ARG
    fs = Dictionary.parse("laplacianSchemes { default Gauss linear corrected; laplacian(a,b) Gauss linear limited 0.5; }"
                          "divSchemes { default bounded Gauss upwind; }")
    assert scheme(fs, "laplacianSchemes", "laplacian(k,T)") == abi.SCHEME_CORRECTED
    for sec, name in (("laplacianSchemes", "laplacian(a,b)"), ("divSchemes", "div(phi,T)")):
        with pytest.raises(abi.FvgbError) as e:
            scheme(fs, sec, name)
        assert e.value.status == abi.ERR_UNSUPPORTED


def test_syntax():
    d = Dictionary.parse("""
        a 1; b 2.5; c (1 2 3); w "quoted string"; s yes;
        base { x 1; y 2; }
        derived { $base; y 3; }   // merged, then y replaced
        v $b;                     /* a value variable */
        "(U|k|epsilon)" { solver PBiCGStab; }
        U { solver PCG; }
        list ((0 0 0) (1 0 0));
        m { p 1; }
        m { q 2; }                // a repeated sub-dictionary merges
        a 7;                      // a repeated primitive entry replaces
        #remove b
    """)
    assert d.get("a") == 7 and "b" not in d
    assert d.get("c") == (1.0, 2.0, 3.0)
    assert d.get("w") == "quoted string"
    assert d.get_bool("s") is True
    assert d.subDict("derived").get("x") == 1 and d.subDict("derived").get("y") == 3
    assert d.subDict("base").get("y") == 2
    assert d.get("v") == 2.5
    assert d.subDict("k").get("solver") == "PBiCGStab"   # pattern match
    assert d.subDict("U").get("solver") == "PCG"          # a plain keyword wins over a pattern
    assert d.get("list") == ["(", "(", 0, 0, 0, ")", "(", 1, 0, 0, ")", ")"]
    assert sorted(d.subDict("m").keys()) == ["p", "q"]
    # scopes: $name inside a sub-dictionary finds the enclosing entry
    d = Dictionary.parse("tol 1e-6; solvers { p { tolerance $tol; } }")
    assert d.subDict("solvers").subDict("p").get("tolerance") == 1e-6
    # the text writer gives a dictionary that reads back the same
    again = Dictionary.parse(d.text())
    assert again.subDict("solvers").subDict("p").get("tolerance") == 1e-6


def test_insert_and_copy():
    d = Dictionary.empty()
    d.insert("solver", "PCG")
    d.insert("type", "solver::Cg")   # not a plain word: stored quoted
    d.insert("tol", 1e-6)
    d.insert("n", 3)
    d.insert("v", (1.0, 2.0, 3.0))
    sub = Dictionary.parse("x 1;")
    d.insert("sub", sub)
    c = d.copy()
    d.remove("solver")
    assert "solver" in c and "solver" not in d
    assert c.get("type") == "solver::Cg" and c.get("tol") == 1e-6 and c.get("n") == 3
    assert c.get("v") == (1.0, 2.0, 3.0) and c.subDict("sub").get("x") == 1
    e = c.insert_dict("criteria")
    e.insert("iteration", 5)
    assert c.subDict("criteria").get("iteration") == 5


@pytest.mark.parametrize("text,status", [
    ("a 1", abi.ERR_INVALID_ARG),            # no ';'
    ("a { b 1;", abi.ERR_INVALID_ARG),       # no '}'
    ("a 1; }", abi.ERR_INVALID_ARG),         # stray '}'
    ("a $missing;", abi.ERR_INVALID_ARG),    # undefined variable
    ("a \"open;", abi.ERR_INVALID_ARG),      # unterminated string
    ("#calc \"1+2\";", abi.ERR_UNSUPPORTED),
    ("#include \"no_such_file\"", abi.ERR_INVALID_ARG),
])
def test_syntax_errors(text, status):
    with pytest.raises(abi.FvgbError) as e:
        Dictionary.parse(text)
    assert e.value.status == status


def test_include_if_present_and_nesting(tmp_path):
    (tmp_path / "inc").write_text("x 3;\n")
    (tmp_path / "loop").write_text('#include "loop"\n')
    d = Dictionary.parse('#includeIfPresent "absent"\n#include "inc"\ny $x;', include_dir=tmp_path)
    assert d.get("y") == 3
    with pytest.raises(abi.FvgbError):
        Dictionary.read(tmp_path / "loop")


def test_cpp_facade_dictionary(ref):
    """fvgb_neon.hpp's Dictionary / mapFvSolution / solverConfig, compiled and
    run on the host (the reference's readDict and compatibility checks)."""
    import subprocess
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    out = root / "tests" / "cpp" / "_build"
    out.mkdir(parents=True, exist_ok=True)
    exe = out / "dict_adapter"
    lib = root / "foamadapter_gb300" / "_lib"
    cmd = ["g++", "-O1", "-std=c++17", f"-I{root / 'include'}", f"-I{root / 'foamadapter_gb300' / 'adapter'}",
           "-I/usr/local/cuda/include", str(root / "tests" / "cpp" / "dict_adapter.cpp"), "-o", str(exe),
           f"-L{lib}", "-lfvgb", "-L/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{lib}",
           "-Wl,-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(ref)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_pde_solver_configured_by_fv_solution(cuda, ref):
    """The heat-transfer tutorial's fvSolution (T: PCG, DIC, tolerance 1e-06)
    drives PDESolver.solve: the same iterations and bits as the explicit
    configuration it maps to (whose parity with the oracle the solver tests
    check)."""
    import numpy as np
    import torch

    from foamadapter_gb300 import mesh, neon
    from foamadapter_gb300.mesh import DeviceMesh
    from oracle.pyoracle import Oracle  # the face diffusivity only

    fv = Dictionary.read(ref / "tutorials/heatTranfer3D/system/fvSolution")
    hm = mesh.box(14, 10, 8, jitter=0.1, seed=7)
    dm = DeviceMesh(hm)
    o = Oracle(hm)
    k = np.exp(0.5 * np.random.default_rng(7).standard_normal(hm.n))
    gamma_h = o.interp_linear(1, k, np.ascontiguousarray(k[hm.bcells]))
    gamma = neon.SurfaceField(dm, gamma_h)
    bcs = [("fixedValue", 400.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    results = []
    for how in ("dict", "kwargs"):
        T = neon.VolumeField(dm, np.full(hm.n, 300.0), bcs, name="T")
        old = T.internal.clone()
        eqn = neon.PDESolver([neon.ddt(old), neon.laplacian(gamma, -1.0)], T, 0.01)
        st = eqn.solve(fvSolution=fv) if how == "dict" else eqn.solve(rel_tol=0.0, abs_tol=1e-6, max_iter=1000)
        assert st.status == abi.OK
        results.append((st.num_iter, T.internal.cpu().numpy().copy()))
    assert results[0][0] == results[1][0]
    assert np.array_equal(results[0][1], results[1][1])
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_pde_solver_configured_by_dilu_entry(cuda, ref):
    """The reference's test/setup_advection fvSolution (T: PBiCGStab, DILU,
    tolerance 1e-14, relTol 0) on an implicit upwind convection-diffusion step:
    BiCGStab with the ILU(0) preconditioner, the same iterations and bits as the
    explicit configuration it maps to and as the oracle's restatement."""
    import numpy as np
    import torch

    from foamadapter_gb300 import mesh, neon
    from foamadapter_gb300.mesh import DeviceMesh
    from oracle.pyoracle import Oracle

    fv = Dictionary.read(ref / "test/setup_advection/system/fvSolution")
    hm = mesh.box(16, 12, 10, jitter=0.1, seed=3)
    dm = DeviceMesh(hm)
    o = Oracle(hm)
    U = np.array([1.0, 0.4, -0.2])
    F = neon.SurfaceField(dm, o.flux_vec(np.tile(U, hm.n), np.tile(U, hm.nbf)))
    nu = neon.SurfaceField(dm, np.full(hm.nif + hm.nbf, 1e-3))
    bcs = [("fixedValue", 1.0)] + [("zeroGradient", 0.0)] * (hm.npatch - 1)
    T0 = np.random.default_rng(3).random(hm.n)
    results = []
    for how in ("dict", "kwargs"):
        T = neon.VolumeField(dm, T0, bcs, name="T")
        old = T.internal.clone()
        eqn = neon.PDESolver([neon.ddt(old), neon.div(F, "upwind"), neon.laplacian(nu, -1.0)], T, 0.05)
        if how == "dict":
            st = eqn.solve(fvSolution=fv)
        else:
            st = eqn.solve(rel_tol=0.0, abs_tol=1e-14, max_iter=1000, method=abi.SOLVER_BICGSTAB,
                           preconditioner=abi.PRECOND_ILU)
        assert st.status == abi.OK and st.num_iter > 1
        results.append((st.num_iter, st.final_res_norm, T.internal.cpu().numpy().copy()))
    assert results[0][:2] == results[1][:2]
    assert np.array_equal(results[0][2], results[1][2])
    v, r, _, _ = [t.cpu().numpy() for t in eqn.ls.export()]
    xo = old.cpu().numpy().copy()
    so = o.solve(v, r, xo, rel_tol=0.0, abs_tol=1e-14, max_iter=1000, method=1, preconditioner=2)
    assert (so.status, so.num_iter, so.final_res_norm) == (0, results[1][0], results[1][1])
    assert np.array_equal(xo, results[1][2])
    torch.cuda.synchronize()


def test_ginkgo_json_configs(ref, tmp_path):
    """The reference's own Ginkgo configurations (tutorials/cylinder2D/system/gko)."""
    from foamadapter_gb300.dictionary import ginkgo_config

    gko = ref / "tutorials/cylinder2D/system/gko"
    mg = ginkgo_config(gko / "config.mg.json")
    assert mg["method"] == abi.SOLVER_CG and mg["preconditioner"] == abi.PRECOND_MULTIGRID
    assert mg["max_iter"] == 100 and mg["abs_tol"] == 1e-5 and mg["rel_tol"] == 0.0
    assert mg["flags"] == 0
    for name in ("config.bj.json", "p.config.bj.json"):  # ResidualNorm with Ginkgo's default baseline rhs_norm
        bj = ginkgo_config(gko / name)
        assert bj["method"] == abi.SOLVER_CG and bj["preconditioner"] == abi.PRECOND_JACOBI
        assert bj["max_iter"] == 1000 and bj["rel_tol"] == 1e-5 and bj["abs_tol"] == 0.0
        assert bj["flags"] == abi.SOLVE_RHS_BASELINE  # ||r|| <= 1e-5 ||b||
    (tmp_path / "base.json").write_text(
        '{"type": "solver::Cg", "preconditioner": {"type": "preconditioner::Jacobi", "max_block_size": 1},'
        ' "criteria": [{"type": "ResidualNorm", "reduction_factor": 1e-9, "baseline": "something"}]}')
    with pytest.raises(abi.FvgbError) as e:
        ginkgo_config(tmp_path / "base.json")
    assert e.value.status == abi.ERR_INVALID_ARG
    (tmp_path / "ok.json").write_text(
        '{"type": "solver::Bicgstab", "preconditioner": {"type": "preconditioner::Jacobi", "max_block_size": 1},'
        ' "criteria": [{"type": "Iteration", "max_iters": 77},'
        ' {"type": "ResidualNorm", "reduction_factor": 1e-9, "baseline": "initial_resnorm"}]}')
    c = ginkgo_config(tmp_path / "ok.json")
    assert c["method"] == abi.SOLVER_BICGSTAB and c["max_iter"] == 77 and c["rel_tol"] == 1e-9
    assert c["preconditioner"] == abi.PRECOND_JACOBI
    # solver::Multigrid as the solver, with Pgm levels
    (tmp_path / "mg.json").write_text(
        '{"type": "solver::Multigrid", "mg_level": [{"type": "multigrid::Pgm"}],'
        ' "criteria": [{"type": "Iteration", "max_iters": 60},'
        ' {"type": "ResidualNorm", "reduction_factor": 1e-8, "baseline": "initial_resnorm"}]}')
    c = ginkgo_config(tmp_path / "mg.json")
    assert c["method"] == abi.SOLVER_MULTIGRID and c["max_iter"] == 60 and c["rel_tol"] == 1e-8
    (tmp_path / "ilu.json").write_text(
        '{"type": "solver::Bicgstab", "preconditioner": {"type": "preconditioner::Ilu", "reverse_apply": false,'
        ' "factorization": {"type": "factorization::ParIlu"}}}')
    c = ginkgo_config(tmp_path / "ilu.json")
    assert c["method"] == abi.SOLVER_BICGSTAB and c["preconditioner"] == abi.PRECOND_ILU
    for text, status in (('{"type": "solver::Cg"', abi.ERR_INVALID_ARG),
                         ('{"type": "solver::Gmres", "preconditioner": {"type": "preconditioner::Jacobi", '
                          '"max_block_size": 1}}', abi.ERR_UNSUPPORTED),
                         ('{"type": "solver::Cg", "preconditioner": {"type": "preconditioner::Jacobi", '
                          '"max_block_size": 32}}', abi.ERR_UNSUPPORTED),
                         ('{"type": "solver::Cg"}', abi.ERR_UNSUPPORTED),
                         ('{"type": "solver::Multigrid", "mg_level": [{"type": "multigrid::Uniform"}]}',
                          abi.ERR_UNSUPPORTED),
                         ('{"type": "solver::Multigrid", "preconditioner": {"type": "preconditioner::Jacobi", '
                          '"max_block_size": 1}}', abi.ERR_UNSUPPORTED)):
        (tmp_path / "bad.json").write_text(text)
        with pytest.raises(abi.FvgbError) as e:
            ginkgo_config(tmp_path / "bad.json")
        assert e.value.status == status, text
    # a solver entry naming the file
    entry = Dictionary.parse('configFile "gko/config.mg.json";')
    assert map_fv_solution(entry).keys() == ["configFile"]
    assert solver_config(entry, config_dir=ref / "tutorials/cylinder2D/system")["preconditioner"] == \
        abi.PRECOND_MULTIGRID
    with pytest.raises(ValueError):
        solver_config(entry)
