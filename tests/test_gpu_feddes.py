"""GPU parity of the Feddes root-water uptake (ETRAN, etran.f:6-81): the
CUDA path through the C ABI against the CPU oracle on a hillslope that
evaporates at 1e-6 m/s with SCF = 1 and two vegetation types.

Tolerances as in test_gpu_parity.py: heads within 1e-6 m, step times within
1e-9 s, nonlinear iteration counts equal, linear counts within +-1 (FP64),
per-step mass-balance errors within 1e-8 relative (the reference's mass
balance does not count QTRANIE, so the transpired volume shows up in ERRAS
on both sides).
"""
import numpy as np
import pytest

from test_feddes import FEDDES2, feddes_case

pytestmark = pytest.mark.gpu

RATE = -1e-6
NSTEPS = 25


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
        p, t, dt, st = s.state(0)
        its, sts = s.records(0)
    return p, sts, its


def _check_steps(sts, osr):
    assert len(sts) == len(osr)
    assert [r["iter"] for r in sts] == [r["iter"] for r in osr]
    np.testing.assert_allclose([r["time"] for r in sts], [r["time"] for r in osr],
                               rtol=0, atol=1e-9)


def test_feddes_fp64_picard_matches_oracle():
    case = feddes_case(rate=RATE)
    o = _oracle(case)
    p, sts, its = _gpu(case)
    po, _, _ = o.state()
    osr, oir = o.step_records(), o.iter_records()
    _check_steps(sts, osr)
    assert np.max(np.abs(p - po)) <= 1e-6
    for a, b in zip(sts, osr):
        assert abs(a["erras"] - b["erras"]) <= 1e-8 * max(abs(b["erras"]), 1e-12)
    assert abs(sts[-1]["cerras"] - osr[-1]["cerras"]) <= 1e-8 * abs(osr[-1]["cerras"])
    assert max(abs(a["niter"] - b["niter"]) for a, b in zip(its, oir)) <= 1
    # the sink acts: without it (SCF = 0, evaporation through the surface)
    # the heads differ by centimetres
    p0, _, _ = _gpu(feddes_case(rate=RATE, scf=0.0))
    assert np.max(np.abs(p - p0)) > 1e-2


@pytest.mark.parametrize("graphs", [False, True])
def test_feddes_fp32_column_line_matches_oracle(graphs):
    case = feddes_case(rate=RATE)
    o = _oracle(case)
    case.parm.precond = 2
    p, sts, _ = _gpu(case, precision=1, graphs=graphs)
    po, _, _ = o.state()
    osr = o.step_records()
    _check_steps(sts, osr)
    assert np.max(np.abs(p - po)) <= 1e-6
    assert abs(sts[-1]["cerras"] - osr[-1]["cerras"]) <= 1e-6 * abs(osr[-1]["cerras"])


def test_feddes_newton_has_no_sink_like_the_reference():
    """BCNEW (bcnew.f) does not subtract QTRANIE: with SCF = 1 the Newton
    scheme loses the evaporation altogether, on both sides."""
    case = feddes_case(rate=RATE, iopt=2)
    o = _oracle(case)
    p, sts, _ = _gpu(case)
    po, _, _ = o.state()
    _check_steps(sts, o.step_records())
    assert np.max(np.abs(p - po)) <= 1e-6


def test_feddes_batch_gates_the_sink_per_member():
    """A batch of a vegetated member (SCF = 1) and a bare one (SCF = 0)
    reproduces the two single-member oracle runs."""
    from pycathy_wrapper_gb300.api import Simulation
    cases = [feddes_case(rate=RATE), feddes_case(rate=RATE, scf=0.0, feddes=None,
                                                 root_map=None)]
    for c in cases:
        c.parm.precond = 2
    with Simulation(cases, precision=1) as s:
        for _ in range(NSTEPS):
            s.step()
        heads = [s.state(m)[0] for m in range(2)]
        recs = [s.records(m)[1] for m in range(2)]
    for c, p, sts in zip(cases, heads, recs):
        c.parm.precond = 0
        o = _oracle(c)
        _check_steps(sts, o.step_records())
        assert np.max(np.abs(p - o.state()[0])) <= 1e-6


def test_feddes_inputs_are_checked(capfd):
    """Refused with EINVAL and the reason on stderr."""
    from pycathy_wrapper_gb300.api import Simulation
    deep = FEDDES2.copy()
    deep[1, 3] = 2.5  # ZROOT below the 2 m deep bottom nodes
    with pytest.raises(RuntimeError, match="invalid argument"):
        Simulation(feddes_case(rate=RATE, feddes=deep))
    assert "ZROOT reaches the bottom node" in capfd.readouterr().err
    with pytest.raises(RuntimeError, match="invalid argument"):
        Simulation(feddes_case(rate=RATE, feddes=None))
    assert "Feddes table" in capfd.readouterr().err
