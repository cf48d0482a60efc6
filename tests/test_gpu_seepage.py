"""GPU parity of the seepage faces (sfinit.f, extall.f, bkpic.f, fluxmb.f,
the ISFCVG test of flow3d.f) through the C ABI against the CPU oracle, on a
hillslope whose lowest edge carries a vertical seepage face per column.

Tolerances: heads within 1e-6 m, step times within 1e-9 s, the exit points
identical, nonlinear iteration counts equal on the FP64 paths; seepage
fluxes and mass-balance errors within 1e-8 relative on the FP64 Picard
path.  The FP32 path is held to the heads and the exit points.
"""
import numpy as np
import pytest

from test_seepage import seepage_case

pytestmark = pytest.mark.gpu

NSTEPS = 40


def _oracle(case, nsteps=NSTEPS):
    import oracle as O
    o = O.Oracle(case)
    for _ in range(nsteps):
        if o.step() != 0:
            break
    return o


def _gpu(case, nsteps=NSTEPS, **kw):
    from pycathy_wrapper_gb300.api import Simulation
    with Simulation(case, **kw) as s:
        for _ in range(nsteps):
            s.step()
        p = s.state(0)[0]
        its, sts = s.records(0)
        ex, q = s.seepage(0)
    return p, sts, its, ex, q


def _check_steps(sts, osr):
    assert len(sts) == len(osr)
    assert [r["iter"] for r in sts] == [r["iter"] for r in osr]
    np.testing.assert_allclose([r["time"] for r in sts], [r["time"] for r in osr],
                               rtol=0, atol=1e-9)


@pytest.mark.parametrize("isfcvg", [1, 0])
def test_seepage_fp64_picard_matches_oracle(isfcvg):
    case = seepage_case(isfcvg=isfcvg)
    o = _oracle(case)
    p, sts, its, ex, q = _gpu(case)
    oex, oq = o.seepage()
    osr, oir = o.step_records(), o.iter_records()
    _check_steps(sts, osr)
    assert np.max(np.abs(p - o.state()[0])) <= 1e-6
    np.testing.assert_array_equal(ex, oex)
    scale = np.abs(oq).max()
    assert scale > 0.0
    assert np.max(np.abs(q - oq)) <= 1e-8 * scale
    for a, b in zip(sts, osr):
        assert abs(a["sfflw"] - b["sfflw"]) <= 1e-8 * max(abs(b["sfflw"]), 1e-12)
        assert abs(a["erras"] - b["erras"]) <= 1e-8 * max(abs(b["vout"]), 1e-12)
    assert max(abs(a["niter"] - b["niter"]) for a, b in zip(its, oir)) <= 1


@pytest.mark.parametrize("graphs", [False, True])
def test_seepage_fp32_column_line_matches_oracle(graphs):
    case = seepage_case()
    o = _oracle(case)
    case.parm.precond = 2
    p, sts, _, ex, _ = _gpu(case, precision=1, graphs=graphs)
    oex, _ = o.seepage()
    osr = o.step_records()
    assert len(sts) == len(osr)
    assert abs(sts[-1]["time"] - osr[-1]["time"]) < 1e-9
    assert np.max(np.abs(p - o.state()[0])) <= 1e-6
    np.testing.assert_array_equal(ex, oex)
    assert abs(sts[-1]["cerras"] - osr[-1]["cerras"]) <= 1e-6 * abs(osr[-1]["cvout"])


def test_seepage_newton_matches_oracle():
    case = seepage_case(iopt=2)
    o = _oracle(case)
    p, sts, _, ex, _ = _gpu(case)
    oex, _ = o.seepage()
    _check_steps(sts, o.step_records())
    assert np.max(np.abs(p - o.state()[0])) <= 1e-6
    np.testing.assert_array_equal(ex, oex)


def test_seepage_member_in_a_batch_with_a_bare_member():
    from pycathy_wrapper_gb300.api import Simulation
    from pycathy_wrapper_gb300.inputs import config0
    cases = [seepage_case(precond=2), config0(tmax=3600.0, precond=2)]
    with Simulation(cases, precision=1) as s:
        for _ in range(NSTEPS):
            s.step()
        heads = [s.state(m)[0] for m in range(2)]
        recs = [s.records(m)[1] for m in range(2)]
        ex, _ = s.seepage(0)
    for c, p, sts in zip(cases, heads, recs):
        c.parm.precond = 0
        o = _oracle(c)
        assert len(sts) == len(o.step_records())
        assert np.max(np.abs(p - o.state()[0])) <= 1e-6
    np.testing.assert_array_equal(ex, _oracle(cases[0]).seepage()[0])


def test_seepage_restart_applies_sfinit():
    """set_state is a new initial condition: SFINIT runs on it."""
    import oracle as O
    from pycathy_wrapper_gb300.api import Simulation
    case = seepage_case()
    o = O.Oracle(case)
    o2 = O.Oracle(seepage_case(wt=0.6))
    p0 = o2.state()[0]
    # the heads of the shallower water table before its SFINIT
    nodes = np.concatenate(case.bc.sfnod) - 1
    ex2, _ = o2.seepage()
    z = o2.mesh()["z"]
    p_ic = p0.copy()
    p_ic[nodes] = (z[nodes % o2.nnod] - z[nodes] - 0.6)
    o.set_state(p_ic, 10.0, 10.0)
    for _ in range(10):
        o.step()
    with Simulation(case) as s:
        s.set_state(0, p_ic, 10.0, 10.0)
        exs, _ = s.seepage(0)
        np.testing.assert_array_equal(exs, ex2)
        for _ in range(10):
            s.step()
        p = s.state(0)[0]
        ex, _ = s.seepage(0)
    assert np.max(np.abs(p - o.state()[0])) <= 1e-6
    np.testing.assert_array_equal(ex, o.seepage()[0])


def test_seepage_inputs_are_checked(capfd):
    from pycathy_wrapper_gb300.api import Simulation
    case = seepage_case()
    case.bc.sfnod[0] = case.bc.sfnod[0][::-1].copy()
    with pytest.raises(RuntimeError, match="invalid argument"):
        Simulation(case)
    assert "descending elevation" in capfd.readouterr().err
    case = seepage_case()
    case.bc.sfnod[2] = case.bc.sfnod[1].copy()
    with pytest.raises(RuntimeError, match="invalid argument"):
        Simulation(case)
    assert "repeated" in capfd.readouterr().err
