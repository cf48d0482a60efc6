"""Parity of the benchmarked path against the oracle at bench scale.

The bench runs the 256-member ensemble (seeds 1000+m) for one simulated day
on the FP32 batched path: FP32 assembly and column-line-preconditioned FP32
PCG inside the FP64 residual loop, one CUDA graph per Picard iteration.
These tests run that exact path (``Simulation(cases, precision=1,
graphs=True)``, ``precond=2``) on real ensemble draws -- four members that finish (1007, 1046, 1053,
1123) and two that fail within the day (1115, 1036: DTMIN reached without
Picard convergence) -- for the full day,
batched together, and compare every member with the CPU oracle running the
reference's method (FP64, IC(0)-PCG) on the same inputs, with the default
FP32 inner tolerance (1e-8).  A config-1-style
member (40x40 fractal DEM, 15 layers, per-cell lognormal Ks) is checked for
the 6-hour rain pulse the same way.  The FP64 path (``precision=0``, IC(0))
is checked iterate for iterate on two of the members, and the CPU-runnable
hillslope configuration for its full simulated day on both paths.  Three of
the draws run again with the Feddes root-water uptake switched on
(``inputs.with_vegetation``).

Tolerances, written where they are asserted:
  * heads: max |psi_gpu - psi_oracle| <= 1e-6 m at the end of the run;
  * time steps: the same number of accepted steps at the same times
    (1e-9 s), Picard iteration counts equal at >= 99 % of the steps (the
    FP32 inner solve may stop one Picard iteration apart where the
    convergence test is decided by round-off, without changing dt);
  * mass balance: cumulative mass-balance error |CERRAS_gpu - CERRAS_orc|
    <= 1e-8 * CVIN for the FP64 path; for the FP32 path the bound is
    1e-7 * CVIN -- its iterates differ from the oracle's by up to 4e-7 m
    (the stopping test decides at different, equally valid iterates), and
    a head difference h changes the stored water by about
    V * C * h (V volume, C specific moisture capacity);
  * members that fail: the GPU fails too, within 0.1 % of the oracle's
    failure time (the last steps run at DTMIN with non-converging Picard
    iterations, where round-off decides the exact step of failure).
"""
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MEMBERS = [7, 46, 53, 123, 115, 36]       # seeds 1000 + m
FAILING = {115, 36}
VEG_MEMBERS = [7, 46, 123]                # the same draws with the Feddes sink
FP64_MEMBERS = [46, 36]
DAY = 86400.0


def _oracle_job(args):
    kind, idx, tmax = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from pycathy_wrapper_gb300 import inputs as I
    if kind == "c2":
        c = I.config2_members(256, tmax=tmax)[idx]
        c.parm.precond = 0
    elif kind == "veg":
        c = I.with_vegetation(I.config2_members(256, tmax=tmax)[idx])
        c.parm.precond = 0
    else:
        c = I.config1(ncell=40, nstr=15, tmax=tmax)
    o = O.Oracle(c)
    rc = o.run()
    return dict(rc=int(rc), p=o.state()[0], steps=o.step_records(),
                iters=[r["iter"] for r in o.step_records()],
                niter=[r["niter"] for r in o.iter_records()])


@pytest.fixture(scope="module")
def oracle_runs():
    ctx = mp.get_context("spawn")  # the test process may already hold a GPU context
    jobs = ([("c2", m, DAY) for m in MEMBERS] + [("c1", 0, 21600.0)] +
            [("veg", m, DAY) for m in VEG_MEMBERS])
    with ctx.Pool(processes=len(jobs)) as pool:
        res = pool.map(_oracle_job, jobs)
    return {(k, m): r for (k, m, _), r in zip(jobs, res)}


def _gpu(cases, **kw):
    from pycathy_wrapper_gb300.api import Simulation
    out = []
    with Simulation(cases, **kw) as s:
        s.run()
        for m in range(len(cases)):
            p, t, dt, st = s.state(m)
            its, sts = s.records(m)
            out.append(dict(p=p, status=st, steps=sts, iters=[r["iter"] for r in sts],
                            niter=[r["niter"] for r in its]))
    return out


def _check_finished(g, o, head_tol, mbe_tol, iter_frac):
    gs, os_ = g["steps"], o["steps"]
    assert g["status"] == 1 and o["rc"] == len(os_)
    assert len(gs) == len(os_)
    np.testing.assert_allclose([r["time"] for r in gs], [r["time"] for r in os_],
                               rtol=0, atol=1e-9 * DAY)
    same = np.mean(np.array(g["iters"]) == np.array(o["iters"]))
    assert same >= iter_frac, same
    assert np.max(np.abs(g["p"] - o["p"])) <= head_tol
    assert abs(gs[-1]["cerras"] - os_[-1]["cerras"]) <= mbe_tol * abs(os_[-1]["cvin"])


def _check_failed(g, o):
    assert g["status"] == 2 and o["rc"] == -1
    tg, to = g["steps"][-1]["time"], o["steps"][-1]["time"]
    assert abs(tg - to) <= 1e-3 * to, (tg, to)


def test_bench_path_full_day_matches_oracle(oracle_runs):
    from pycathy_wrapper_gb300.inputs import config2_members
    allc = config2_members(256, tmax=DAY)
    cases = [allc[m] for m in MEMBERS]
    for c in cases:
        c.parm.precond = 2
    got = _gpu(cases, precision=1, graphs=True)
    for m, g in zip(MEMBERS, got):
        o = oracle_runs[("c2", m)]
        if m in FAILING:
            _check_failed(g, o)
        else:
            _check_finished(g, o, head_tol=1e-6, mbe_tol=1e-7, iter_frac=0.99)


def test_bench_path_heterogeneous_ks_member_matches_oracle(oracle_runs):
    from pycathy_wrapper_gb300.inputs import config1
    c = config1(ncell=40, nstr=15, tmax=21600.0)
    c.parm.precond = 2
    g = _gpu([c], precision=1, graphs=True)[0]
    o = oracle_runs[("c1", 0)]
    _check_finished(g, o, head_tol=1e-6, mbe_tol=1e-7, iter_frac=0.99)


def test_bench_path_vegetated_members_match_oracle(oracle_runs):
    """Three of the draws with the Feddes root-water uptake switched on (SCF
    = 1, grass and shrubs, rain then evaporation) on the bench path for the
    full day; the transpired volume is part of CERRAS on both sides."""
    from pycathy_wrapper_gb300.inputs import config2_members, with_vegetation
    allc = config2_members(256, tmax=DAY)
    cases = [with_vegetation(allc[m]) for m in VEG_MEMBERS]
    for c in cases:
        c.parm.precond = 2
    got = _gpu(cases, precision=1, graphs=True)
    for m, g in zip(VEG_MEMBERS, got):
        _check_finished(g, oracle_runs[("veg", m)], head_tol=1e-6, mbe_tol=1e-7,
                        iter_frac=0.99)


def test_fp64_path_matches_oracle_iterate_for_iterate(oracle_runs):
    from pycathy_wrapper_gb300.inputs import config2_members
    allc = config2_members(256, tmax=DAY)
    cases = [allc[m] for m in FP64_MEMBERS]
    for c in cases:
        c.parm.precond = 0
    got = _gpu(cases, precision=0)
    for m, g in zip(FP64_MEMBERS, got):
        o = oracle_runs[("c2", m)]
        if m in FAILING:
            # the batched FP64 dot products are summed in a launch-dependent
            # order: a member that fails (non-converging iterations at DTMIN)
            # may fail a step apart; status and failure time must agree
            _check_failed(g, o)
            continue
        assert g["iters"] == o["iters"]
        assert g["niter"] == o["niter"]  # same PCG iteration counts
        assert len(g["steps"]) == len(o["steps"])
        assert np.max(np.abs(g["p"] - o["p"])) <= 1e-8
        assert abs(g["steps"][-1]["cerras"] - o["steps"][-1]["cerras"]) <= \
            1e-8 * abs(o["steps"][-1]["cvin"])


def test_config0_hillslope_full_day_matches_oracle():
    """The CPU-runnable configuration for its stated simulated day (20x20
    hillslope, 10 layers, constant rain, Picard + Jacobi-PCG, dt 1..600 s):
    the FP64 path with the reference's preconditioner iterate for iterate,
    and the benchmarked FP32 column-line path step for step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from pycathy_wrapper_gb300.inputs import config0
    o = O.Oracle(config0(tmax=DAY, precond=1))
    assert o.run() > 0
    orc = dict(rc=len(o.step_records()), p=o.state()[0], steps=o.step_records(),
               iters=[r["iter"] for r in o.step_records()],
               niter=[r["niter"] for r in o.iter_records()])
    g64 = _gpu([config0(tmax=DAY, precond=1)], precision=0)[0]
    assert g64["iters"] == orc["iters"] and g64["niter"] == orc["niter"]
    _check_finished(g64, orc, head_tol=1e-8, mbe_tol=1e-8, iter_frac=1.0)
    g32 = _gpu([config0(tmax=DAY, precond=2)], precision=1, graphs=True)[0]
    _check_finished(g32, orc, head_tol=1e-6, mbe_tol=1e-7, iter_frac=0.99)
