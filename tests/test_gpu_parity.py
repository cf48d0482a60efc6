"""GPU parity: the CUDA path through the C ABI against the CPU oracle and the
reference's golden first iteration.

Tolerances: heads within 1e-6 m (the spec bar, TOLUNS = 1e-6 for the
synthetic configurations), relative mass-balance errors within 1e-8 of the
oracle's, linear-solver iteration counts equal for the FP64 path (same
recurrences and preconditioner), within +-1 where round-off decides a stop.
"""
import numpy as np
import pytest

from conftest import golden_json, load_golden_case

pytestmark = pytest.mark.gpu


def _sim(case, **kw):
    from pycathy_wrapper_gb300.api import Simulation
    return Simulation(case, **kw)


@pytest.mark.parametrize("key", ["weill", "soil3d", "etp", "eo", "da2"])
def test_first_iteration_matches_reference_golden(key):
    g = golden_json()[key]
    case = load_golden_case(key)
    with _sim(case) as s:
        s.step()
        its, _ = s.records(0)
    r = its[0]
    fi, lin = g["first_iter"], g["linear"]
    assert r["niter"] == fi["niter"]
    assert r["ikmax"] == fi["ikmax"]
    for k in ("pl2", "pinf", "fl2", "finf"):
        assert abs(r[k] - fi[k]) / abs(fi[k]) < 6e-4, (k, r[k], fi[k])
    # the PCG's last residual: to 1e-4 where the system is well scaled; the
    # evaporation run's only forcing is the Feddes sink (|RHS| ~ 1e-7), and
    # its 28th residual (4.8e-11) moves by about 1 % with the order of the
    # parallel FP64 dot products (the serial oracle matches it to 2e-6)
    lin_tol = 5e-2 if key == "etp" else 1e-4
    if lin is not None:
        assert abs(r["lin_err"] - lin["err"]) / lin["err"] < lin_tol


@pytest.mark.parametrize("key", ["weill", "soil3d"])
def test_picard_system_matches_oracle(key):
    import oracle as O
    case = load_golden_case(key)
    o = O.Oracle(case)
    c1, tn, xt5, dm = o.picard_system()
    with _sim(case) as s:
        vals, rhs, xt5g, dmg = s.picard_system(0)
        m = s.mesh(0)
    n = o.n
    om = o.mesh()
    topol, ja = om["topol"], om["ja"]
    rows = np.repeat(np.arange(n), np.diff(topol))
    up = {(i, j - 1): c1[k] for k, (i, j) in enumerate(zip(rows, ja))}
    grow = np.repeat(np.arange(n), np.diff(m["rowptr"]))
    ref = np.array([up[(i, j)] if (i, j) in up else up[(j, i)] for i, j in zip(grow, m["cols"])])
    scale = np.abs(ref).max()
    assert np.max(np.abs(vals - ref)) <= 1e-10 * scale
    np.testing.assert_array_equal(dmg, dm)
    # the RHS is a sum of stiffness*head terms that cancel (hydrostatic
    # balance): bound by the size of those terms, not of the result
    term = scale * max(1.0, float(np.abs(o.state()[0]).max()))
    assert np.max(np.abs(rhs - tn)) <= 1e-12 * term
    assert np.max(np.abs(xt5g - xt5)) <= 1e-12 * term


def _run_both(case, nsteps, **kw):
    import oracle as O
    o = O.Oracle(case)
    for _ in range(nsteps):
        if o.step() != 0:
            break
    with _sim(case, **kw) as s:
        for _ in range(nsteps):
            s.step()
        p, t, dt, st = s.state(0)
        its, sts = s.records(0)
    po, to, dto = o.state()
    return o, (p, t, sts, its), (po, o.step_records(), o.iter_records())


@pytest.mark.parametrize("precond", [0, 1])
def test_hillslope_steps_match_oracle(precond):
    from pycathy_wrapper_gb300.inputs import config0
    case = config0(tmax=3600.0, precond=precond)
    o, (p, t, sts, its), (po, osr, oir) = _run_both(case, 25)
    assert len(sts) == len(osr)
    assert [r["iter"] for r in sts] == [r["iter"] for r in osr]
    np.testing.assert_allclose([r["time"] for r in sts], [r["time"] for r in osr], rtol=0, atol=1e-9)
    assert np.max(np.abs(p - po)) <= 1e-6
    for a, b in zip(sts, osr):
        assert abs(a["errel"] - b["errel"]) <= 1e-8 * max(1.0, abs(b["errel"])) + 1e-8
        assert abs(a["dstore"] - b["dstore"]) <= 1e-8 * max(abs(b["dstore"]), 1e-12)
    dn = [abs(a["niter"] - b["niter"]) for a, b in zip(its, oir)]
    assert max(dn) <= 1


def test_hillslope_indp3_initial_condition_matches_oracle():
    """INDP = 3 (water table 1.5 m above each column's bottom node,
    icvhwt.f) through the engine, against the oracle over 10 steps."""
    from pycathy_wrapper_gb300.inputs import config0
    case = config0(tmax=3600.0, precond=0)
    case.bc.indp, case.bc.wtposition = 3, 1.5
    o, (p, t, sts, its), (po, osr, oir) = _run_both(case, 10)
    assert len(sts) == len(osr)
    np.testing.assert_allclose([r["time"] for r in sts], [r["time"] for r in osr], rtol=0, atol=1e-9)
    assert np.max(np.abs(p - po)) <= 1e-6


def test_hillslope_column_line_preconditioner_matches_oracle_heads():
    from pycathy_wrapper_gb300.inputs import config0
    import oracle as O
    case = config0(tmax=3600.0, precond=0)
    o = O.Oracle(case)
    for _ in range(25):
        o.step()
    case2 = config0(tmax=3600.0, precond=2)
    with _sim(case2) as s:
        for _ in range(25):
            s.step()
        p, t, dt, st = s.state(0)
        _, sts = s.records(0)
    po, to, _ = o.state()
    assert abs(sts[-1]["time"] - o.step_records()[-1]["time"]) < 1e-9
    assert np.max(np.abs(p - po)) <= 1e-6


def test_mixed_precision_heads_within_tolerance():
    from pycathy_wrapper_gb300.inputs import config0
    import oracle as O
    case = config0(tmax=3600.0, precond=0)
    o = O.Oracle(case)
    for _ in range(25):
        o.step()
    case2 = config0(tmax=3600.0, precond=2)
    with _sim(case2, precision=1) as s:
        for _ in range(25):
            s.step()
        p, t, dt, st = s.state(0)
        _, sts = s.records(0)
    po, to, _ = o.state()
    assert abs(sts[-1]["time"] - o.step_records()[-1]["time"]) < 1e-9
    assert np.max(np.abs(p - po)) <= 1e-6
    osr = o.step_records()
    # the FP32 path stops its Picard iterations at different (valid) iterates
    # than the FP64 reference; its cumulative mass-balance error then differs
    # by a small fraction of the error itself
    assert abs(sts[-1]["cerras"] - osr[-1]["cerras"]) <= 1e-6 * abs(osr[-1]["cvin"])


def test_symslv_dropin_matches_oracle():
    import oracle as O
    from pycathy_wrapper_gb300.api import symslv
    case = load_golden_case("weill")
    o = O.Oracle(case)
    c1, tn, xt5, dm = o.picard_system()
    om = o.mesh()
    noddir = np.nonzero(dm)[0] + 1
    c1p = c1.copy()
    c1p[om["topol"][noddir - 1] - 1] = 1.7e91  # BCPIC penalty as the Fortran caller passes it
    xo, no, eo, ro = O.symslv(om["topol"], om["ja"], c1p, tn, noddir)
    xg, ng, eg, rg, coef2 = symslv(om["topol"], om["ja"], c1p, tn, noddir)
    assert abs(ng - no) <= 1
    assert np.max(np.abs(xg - xo)) <= 1e-8 * np.max(np.abs(xo))
    assert rg < 1e-9


@pytest.mark.parametrize("isolv", [0, -5])
def test_nsyslv_dropin_matches_oracle(isolv):
    import oracle as O
    from pycathy_wrapper_gb300.api import nsyslv
    case = load_golden_case("soil3d")
    o = O.Oracle(case)
    c1, tn, xt5, dm = o.picard_system()
    om = o.mesh()
    n = o.n
    rows = np.repeat(np.arange(n), np.diff(om["topol"]))
    cols = om["ja"] - 1
    import scipy.sparse as sp
    U = sp.csr_matrix((c1, (rows, cols)), shape=(n, n))
    A = (U + U.T - sp.diags(U.diagonal())).tocsr()
    A.sort_indices()
    noddir = np.nonzero(dm)[0] + 1
    A = A.tolil()
    for d in noddir - 1:
        A[d, d] = 1.7e91
    A = A.tocsr()
    A.sort_indices()
    topol = (A.indptr + 1).astype(np.int32)
    ja = (A.indices + 1).astype(np.int32)
    xo, no, eo, ro = O.nsyslv(topol, ja, A.data, tn, noddir, isolv=isolv)
    xg, ng, eg, rg = nsyslv(topol, ja, A.data, tn, noddir, isolv=isolv)
    assert abs(ng - no) <= 1
    assert np.max(np.abs(xg - xo)) <= 1e-7 * np.max(np.abs(xo))


def test_newton_ponded_steps_match_oracle():
    """Newton + ILU(0)-BiCGSTAB (FP64) on the ponded clay loam for 24 steps:
    the same Newton iterations per step, the same BiCGSTAB iteration counts
    (GCSTAS's recurrences and stopping rule; +-1 where round-off decides a
    stop) and heads within 1e-6 m."""
    from pycathy_wrapper_gb300.inputs import config4_member
    case = config4_member(ncell=12, nstr=8, tmax=3600.0)
    o, (p, t, sts, its), (po, osr, oir) = _run_both(case, 24)
    assert [r["iter"] for r in sts] == [r["iter"] for r in osr]
    dn = [abs(a["niter"] - b["niter"]) for a, b in zip(its, oir)]
    assert len(its) == len(oir) and max(dn) <= 1
    assert np.max(np.abs(p - po)) <= 1e-6


@pytest.mark.parametrize("isolv", [0, -5])
def test_newton_fp32_krylov_matches_oracle(isolv):
    """FP32 BiCGSTAB inside the FP64 Newton loop (precision=1, IOPT=2): the
    Jacobian and the residual are assembled in FP64, the correction is
    solved in FP32 (ILU(0) or Jacobi preconditioning), the Newton update,
    convergence test and mass balance stay FP64.  Same Newton iterations per
    step and heads within 1e-6 m of the FP64 oracle."""
    from pycathy_wrapper_gb300.inputs import config4_member
    case = config4_member(ncell=12, nstr=8, tmax=3600.0)
    case.parm.isolv = isolv
    o, (p, t, sts, its), (po, osr, oir) = _run_both(case, 24, precision=1)
    assert len(sts) == len(osr)
    assert [r["iter"] for r in sts] == [r["iter"] for r in osr]
    assert abs(sts[-1]["time"] - osr[-1]["time"]) < 1e-9
    assert np.max(np.abs(p - po)) <= 1e-6
    assert abs(sts[-1]["cerras"] - osr[-1]["cerras"]) <= 1e-6 * abs(osr[-1]["cvin"])


def test_ensemble_batch_matches_single_runs():
    from pycathy_wrapper_gb300.inputs import config2_members
    import oracle as O
    cases = config2_members(3, tmax=1200.0, min_cells=8, max_cells=14)
    for c in cases:
        c.parm.precond = 0
    with _sim(cases) as s:
        s.run()
        got = [s.state(m) for m in range(3)]
        recs = [s.records(m)[1] for m in range(3)]
    for m, c in enumerate(cases):
        o = O.Oracle(c)
        o.run()
        po, to, _ = o.state()
        osr = o.step_records()
        assert len(recs[m]) == len(osr)
        assert abs(recs[m][-1]["time"] - osr[-1]["time"]) < 1e-9
        assert np.max(np.abs(got[m][0] - po)) <= 1e-6


def test_graph_path_matches_kernel_by_kernel_path():
    """The FP32 path run as one CUDA graph per Picard iteration (PCG loop as
    a device-driven conditional node) takes the same steps and iterations
    and reaches the same heads as the kernel-by-kernel path."""
    from pycathy_wrapper_gb300.inputs import config2_members
    cases = config2_members(4, tmax=3600.0, min_cells=8, max_cells=16)
    for c in cases:
        c.parm.precond = 2
    out = {}
    for graphs in (False, True):
        with _sim(cases, precision=1, graphs=graphs) as s:
            s.run()
            out[graphs] = [(s.state(m), s.records(m)) for m in range(len(cases))]
    for m in range(len(cases)):
        (pa, ta, _, sa), (ia, ra) = out[False][m]
        (pb, tb, _, sb), (ib, rb) = out[True][m]
        assert sa == sb == 1 and ta == tb
        assert [r["iter"] for r in ra] == [r["iter"] for r in rb]
        assert [r["niter"] for r in ia] == [r["niter"] for r in ib]
        assert np.max(np.abs(pa - pb)) <= 1e-9
        assert abs(ra[-1]["cerras"] - rb[-1]["cerras"]) <= 1e-9 * max(abs(ra[-1]["cvin"]), 1e-30)


@pytest.mark.parametrize("precision", [0, 1])
def test_chord_slope_kslope1_matches_oracle(precision):
    """KSLOPE=1 (CHPIC1, chpic1.f:25-48): the storage coefficient is the
    chord slope of Se between PTOLD and PTNEW.  TOLKSL is lowered so that
    the chord branch is taken at most nodes of the hillslope's iterations."""
    from pycathy_wrapper_gb300.inputs import config0
    import oracle as O
    case = config0(tmax=3600.0, precond=0)
    case.soil.kslope, case.soil.tolksl = 1, 1e-7
    o = O.Oracle(case)
    for _ in range(20):
        o.step()
    base = config0(tmax=3600.0, precond=0)
    o0 = O.Oracle(base)
    for _ in range(20):
        o0.step()
    gcase = config0(tmax=3600.0, precond=0 if precision == 0 else 2)
    gcase.soil.kslope, gcase.soil.tolksl = 1, 1e-7
    with _sim(gcase, precision=precision) as s:
        for _ in range(20):
            s.step()
        p, t, dt, st = s.state(0)
        its, sts = s.records(0)
    po, to, _ = o.state()
    # the chord branch changes the solution path (else the test is vacuous)
    assert np.max(np.abs(po - o0.state()[0])) > 1e-9 or \
        [r["iter"] for r in o.step_records()] != [r["iter"] for r in o0.step_records()]
    assert abs(sts[-1]["time"] - o.step_records()[-1]["time"]) < 1e-9
    assert [r["iter"] for r in sts] == [r["iter"] for r in o.step_records()]
    assert np.max(np.abs(p - po)) <= 1e-6


def test_newton_chord_slope_kslope1_matches_oracle():
    """KSLOPE=1 on the Newton branch (CHNEW1, chnew1.f:27-53): chord slopes
    of the storage, its derivative and kr under ponded infiltration."""
    from pycathy_wrapper_gb300.inputs import config4_member
    case = config4_member(ncell=12, nstr=8, tmax=600.0)
    case.soil.kslope, case.soil.tolksl = 1, 1e-3
    o, (p, t, sts, its), (po, osr, oir) = _run_both(case, 8)
    assert [r["iter"] for r in sts] == [r["iter"] for r in osr]
    assert np.max(np.abs(p - po)) <= 1e-6


def test_staged_spmv_gives_the_same_heads():
    """The stream SpMV's staged form (each warp copies its next map entry's
    values and columns into shared memory while it multiplies the current
    one) runs for work sets of more than two entries per warp of a resident
    wave; at the same grid (5 blocks per SM) its products and dot products
    are formed in the same order as the direct form's, so the heads are
    bit-identical."""
    from pycathy_wrapper_gb300.inputs import config2_members
    cases = config2_members(4, tmax=900.0, min_cells=40, max_cells=50)
    for c in cases:
        c.parm.precond = 2
    runs = []
    for staged in (0, 1):
        with _sim(cases, precision=1, graphs=True) as s:
            assert sum(z["n"] for z in s.sizes) > 2 * 8 * 152 * 16  # the large-set path
            s.set_schedule(10, 5, 2, staged)
            s.run()
            runs.append([(s.state(m)[0], [r["iter"] for r in s.records(m)[1]])
                         for m in range(len(cases))])
    for (pa, ia), (pb, ib) in zip(*runs):
        assert ia == ib
        np.testing.assert_array_equal(pa, pb)


def test_every_autotuner_schedule_gives_the_same_heads():
    """The autotuner picks the assembly kernel's resident blocks per SM and
    whether its records, columns and gather lists are read directly or
    staged in shared memory by bulk copies, with 16 or 8 lanes per row (the
    same arithmetic in the same order, so bit-identical systems), and the
    stream SpMV's grid
    (which only regroups its FP32 dot products).  Every schedule must reach
    the same heads; the tuner returns one of its candidates and reuses its
    cached choice."""
    from pycathy_wrapper_gb300.inputs import config2_members
    cases = config2_members(3, tmax=1800.0, min_cells=8, max_cells=14)
    for c in cases:
        c.parm.precond = 2
    runs = {}
    scheds = [(a, 8, st) for st in (0, 1) for a in (5, 6, 7, 8)] + \
        [(a, 8, 2) for a in (6, 8, 10, 12)] + [(6, 4, 0), (6, 6, 0)]
    for asm, spmv, staged in scheds:
        with _sim(cases, precision=1, graphs=True) as s:
            s.set_schedule(asm, spmv, staged)
            s.run()
            runs[(asm, spmv, staged)] = [(s.state(m)[0], [r["iter"] for r in s.records(m)[1]])
                                         for m in range(len(cases))]
    base = runs[(6, 8, 0)]
    for key, got in runs.items():
        for (pa, ia), (pb, ib) in zip(base, got):
            assert ia == ib, key
            if key[1] == 8:
                np.testing.assert_array_equal(pa, pb)   # assembly variants: bit-identical
            else:
                assert np.max(np.abs(pa - pb)) <= 1e-9, key
    with _sim(cases, precision=1, graphs=True) as s:
        s.run(5)
        t = s.autotune(5)
        assert t["asm_blocks"] in (5, 6, 7, 8, 10, 12) and t["spmv_blocks"] in (4, 5, 6, 8)
        assert t["asm_ms"] > 0 and t["spmv_ms"] > 0
        again = s.autotune(0)  # the cached choice
        assert (again["asm_blocks"], again["spmv_blocks"], again["asm_staged"],
                again["spmv_staged"]) == (t["asm_blocks"], t["spmv_blocks"], t["asm_staged"],
                                          t["spmv_staged"])
        s.run()
        assert all(s.state(m)[3] == 1 for m in range(len(cases)))


@pytest.mark.parametrize("key,nsteps", [("eo", None), ("eoc", 1500)])
def test_stored_run_matches_reference_records(key, nsteps):
    """The EO-dataset projects' stored runs (every iter record and mbeconv
    row of the steps run, see test_oracle_golden.py) on the FP64 path
    through the C ABI, at the records' printed precision."""
    from test_oracle_golden import _run_records, check_stored_run
    case = load_golden_case(key)
    _, _, _, mb = _run_records(key)
    with _sim(case) as s:
        for _ in range(len(mb) if nsteps is None else nsteps):
            s.step()
        its, sts = s.records(0)
    check_stored_run(key, its, sts, nsteps, strict=False)
