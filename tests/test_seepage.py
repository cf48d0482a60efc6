"""Seepage faces (sfvone.f, sfinit.f, extall.f, extcvg.f, the seepage-face
parts of bcpic.f, bkpic.f, fluxmb.f, masbal.f, bkstep.f and the time loop)
in the oracle: initial exit points, the exit-point rules after every
iteration, the mass balance that counts the seepage outflow, the input
checks, and the project reader/writer for ``input/sfbc``.

No stored reference run has seepage faces (every example's sfbc holds
NSF = 0), so these are properties of the restatement, not reference pins.
"""
import numpy as np
import pytest


def seepage_case(nrow=6, ncol=8, nstr=6, rain=5e-6, wt=1.2, isfcvg=1, iopt=1,
                 tmax=7200.0, precond=0):
    """Hillslope rising along x with a vertical seepage face on every
    column of its lowest edge (x = 0), rain 5e-6 m/s, water table 1.2 m
    deep: the bottom nodes of the faces start as exit points and the exit
    points move while the water table rises."""
    from pycathy_wrapper_gb300.inputs import BC, Case, Parm, Soil, hillslope
    dem = hillslope(nrow=nrow, ncol=ncol, nstr=nstr, slope=0.05)
    soil = Soil.homogeneous(nstr, ks=1e-5)
    parm = Parm(iopt=iopt, toluns=1e-6, deltat=10.0, dtmin=0.5, dtmax=120.0, tmax=tmax,
                precond=precond, isfcvg=isfcvg, ituns=20, ituns1=6, ituns2=12)
    nnod = (nrow + 1) * (ncol + 1)
    faces = [np.array([r * (ncol + 1) + 1 + k * nnod for k in range(nstr + 1)], np.int32)
             for r in range(nrow + 1)]
    bc = BC(atmtim=np.array([0.0, 1e9]), atminp=np.array([rain, rain]), indp=4,
            wtposition=wt, sfnod=faces)
    return Case(dem, soil, parm, bc, name="seepage")


def _faces(case):
    return np.concatenate(case.bc.sfnod) - 1


def test_sfinit_exit_points_below_the_water_table():
    import oracle as O
    case = seepage_case()
    o = O.Oracle(case)
    ex, q = o.seepage()
    p, _, _ = o.state()
    mesh = o.mesh()
    nodes = _faces(case)
    z = mesh["z"]
    # the initial heads before SFINIT: water table 1.2 m below the surface
    zs = z[nodes % o.nnod]
    p_ic = zs - z[nodes] - 1.2
    np.testing.assert_array_equal(ex, (p_ic >= 1e-8).astype(np.int32))
    assert ex.sum() > 0 and ex.sum() < len(nodes)
    assert np.all(p[nodes][ex == 1] == 0.0)
    assert not q.any()


def test_exit_points_and_mass_balance_after_a_run():
    import oracle as O
    case = seepage_case()
    o = O.Oracle(case)
    ex0, _ = o.seepage()
    for _ in range(60):
        assert o.step() == 0
    ex, q = o.seepage()
    p, _, _ = o.state()
    nodes = _faces(case)
    # EXTALL after the last iteration: exit points at zero head, the other
    # face nodes unsaturated, no inflow through an exit point
    assert np.all(p[nodes][ex == 1] == 0.0)
    assert np.all(p[nodes][ex == 0] <= 1e-8)
    assert np.all(q[ex == 1] <= 0.0) and np.all(q[ex == 0] == 0.0)
    assert not np.array_equal(ex, ex0)  # the exit points moved
    sr = o.step_records()
    assert all(r["sfflw"] <= 0.0 for r in sr) and sr[-1]["sfflw"] < 0.0
    # VOUT carries the seepage outflow: the cumulative error is a small
    # fraction of it
    vsf = sum(0.5 * r["deltat"] * (a + b) for r, a, b in
              zip(sr, [x["sfflw"] for x in sr], [0.0] + [x["sfflw"] for x in sr[:-1]]))
    assert vsf < 0.0
    assert abs(sr[-1]["cerras"]) < 0.05 * abs(vsf)


def test_exit_point_convergence_check_flag():
    """ISFCVG = 1 only adds a condition; on this case the exit points settle
    within the iterations and both settings give the same run."""
    import oracle as O
    a, b = O.Oracle(seepage_case(isfcvg=1)), O.Oracle(seepage_case(isfcvg=0))
    for _ in range(30):
        a.step(); b.step()
    assert [r["iter"] for r in a.step_records()] == [r["iter"] for r in b.step_records()]
    np.testing.assert_array_equal(a.state()[0], b.state()[0])


def test_oracle_refuses_bad_seepage_faces():
    import oracle as O
    case = seepage_case()
    case.bc.sfnod[0] = case.bc.sfnod[0][::-1].copy()  # ascending elevation
    with pytest.raises(RuntimeError):
        O.Oracle(case)
    case = seepage_case()
    case.bc.contp = case.bc.sfnod[1][-1:].copy()      # also a Dirichlet node
    case.bc.presc = np.zeros(1)
    with pytest.raises(RuntimeError):
        O.Oracle(case)
    case = seepage_case()
    case.bc.sfnod[2] = case.bc.sfnod[1].copy()        # a node on two faces
    with pytest.raises(RuntimeError):
        O.Oracle(case)


def test_project_round_trip_of_seepage_faces(tmp_path):
    from pycathy_wrapper_gb300.project import read_project
    from pycathy_wrapper_gb300.pycathy import write_project
    case = seepage_case()
    write_project(case, str(tmp_path))
    back = read_project(str(tmp_path))
    assert len(back.bc.sfnod) == len(case.bc.sfnod)
    for a, b in zip(back.bc.sfnod, case.bc.sfnod):
        np.testing.assert_array_equal(a, b)
    assert back.parm.isfcvg == 1


def test_project_reader_reads_empty_sfbc():
    from conftest import load_golden_case
    case = load_golden_case("weill")
    assert case.bc.sfnod == []
