"""Feddes root-water uptake (ETRAN, etran.f:6-81) and vegetation types
(datin.f:221-233): the oracle against a loop-by-loop numpy restatement of
etran.f, the project reader on the reference's stored example, and the
oracle's refusals (no Feddes table with SCF > 0, a root zone that reaches
the bottom node)."""
import os

import numpy as np
import pytest

from conftest import load_golden_case

FEDDES2 = np.array([[0.0, -4.0, -150.0, 1.0, 1.0, 1.0],
                    [-0.5, -2.0, -50.0, 0.6, 2.0, 0.5]])


def feddes_case(nrow=8, ncol=8, nstr=6, rate=-5e-8, scf=1.0, wt=1.0, iopt=1,
                tmax=3600.0, feddes=FEDDES2, root_map="halves"):
    """Hillslope with evaporation at ``rate`` [m/s] and two vegetation
    types (left half 1, right half 2)."""
    from pycathy_wrapper_gb300.inputs import BC, Case, Parm, Soil, hillslope
    dem = hillslope(nrow=nrow, ncol=ncol, nstr=nstr)
    rm = None
    if root_map == "halves":
        rm = np.ones((nrow, ncol))
        rm[:, ncol // 2:] = 2.0
    soil = Soil.homogeneous(nstr, scf=scf)
    soil.feddes = feddes
    soil.root_map = rm
    parm = Parm(iopt=iopt, toluns=1e-6, deltat=10.0, dtmin=1.0, dtmax=300.0, tmax=tmax,
                precond=0)
    bc = BC(atmtim=np.array([0.0, 1e9]), atminp=np.array([rate, rate]), indp=4,
            wtposition=wt)
    return Case(dem, soil, parm, bc, name="feddes")


def veg_types(case):
    """VEG_TYPE per surface node: TRIANGOLI's two triangles per cell
    (NW-SW-SE and NW-SE-NE) averaged by TPNODI2D, truncated."""
    d, s = case.dem, case.soil
    nr, nc = d.nrow, d.ncol
    acc = np.zeros((nr + 1, nc + 1))
    cnt = np.zeros((nr + 1, nc + 1))
    rm = np.ones((nr, nc)) if s.root_map is None else np.asarray(s.root_map, float)
    for i in range(nr):
        for j in range(nc):
            v = rm[i, j] * d.factor
            for (a, b), w in (((i, j), 2), ((i + 1, j + 1), 2), ((i + 1, j), 1),
                              ((i, j + 1), 1)):
                acc[a, b] += w * v
                cnt[a, b] += w
    return (acc / cnt).astype(int).reshape(-1)


def etran_ref(pnew, z, atmpot, veg, feddes, nnod, nstr, scf):
    """etran.f:21-79, statement by statement (0-based node k = J*nnod + I)."""
    n = nnod * (nstr + 1)
    q = np.zeros(n)
    btrani = np.zeros(n)
    btran = np.zeros(nnod)
    omg = np.zeros(nnod)
    etp = np.zeros(nnod)
    for i in range(nnod):
        pcana, pcref, pcwlt, zroot, pz, _ = feddes[veg[i] - 1]
        zsurf = z[i]
        depth = 0.0
        etp[i] = -scf * atmpot[i] if atmpot[i] < 0.0 else 0.0
        j = 0
        while depth <= zroot:
            k = j * nnod + i
            s1, s2 = pcana, pcana + 1e-3
            dz = (zsurf - z[k + nnod]) / 2 if j == 0 else (z[k - nnod] - z[k + nnod]) / 2
            gx1 = min(1.0, max(0.0, (pnew[k] - pcwlt) / (pcref - pcwlt)))
            gx2 = min(1.0, max(0.0, 1.0 - (pnew[k] - s1) / (s2 - s1)))
            gx = min(gx1, gx2)
            beta = (1 - depth / zroot) * np.exp(-pz * depth / zroot)
            btrani[k] = max(0.0, beta * dz * gx)
            btran[i] += beta * dz
            omg[i] += gx * beta * dz
            j += 1
            depth = zsurf - z[j * nnod + i]
        btran[i] = max(0.0, btran[i])
        omg[i] = omg[i] / btran[i]
    for i in range(nnod):
        omgc = feddes[veg[i] - 1][5]
        for j in range(nstr + 1):
            k = j * nnod + i
            q[k] = etp[i] * btrani[k] / btran[i] / max(omg[i], omgc)
    return q


def test_oracle_etran_matches_restatement():
    import oracle as O
    case = feddes_case()
    orc = O.Oracle(case)
    mesh = orc.mesh()
    p0, _, dt = orc.state()
    assert orc.step() == 0
    q, vt = orc.qtranie()
    veg = veg_types(case)
    assert np.array_equal(vt, veg)
    assert set(np.unique(vt)) == {1, 2}
    atmpot = case.bc.atminp[0] * mesh["arenod"]
    ref = etran_ref(p0, mesh["z"], atmpot, veg, FEDDES2, orc.nnod, case.dem.nstr, 1.0)
    assert np.count_nonzero(ref) > orc.nnod
    assert np.allclose(q, ref, rtol=1e-13, atol=0.0)
    # the sink removes SCF x the potential evaporation through each column
    col = q.reshape(case.dem.nstr + 1, orc.nnod)
    gx_full = np.isclose(col.sum(axis=0), -atmpot, rtol=1e-12)
    assert gx_full.any()
    assert np.all(col.sum(axis=0) <= -atmpot * (1 + 1e-12))


def test_oracle_etran_zero_without_evaporation_or_scf():
    import oracle as O
    for kw in (dict(rate=2e-8), dict(scf=0.0)):
        orc = O.Oracle(feddes_case(**kw))
        assert orc.step() == 0
        q, _ = orc.qtranie()
        assert not q.any()


def test_oracle_refuses_bad_feddes_inputs():
    import oracle as O
    with pytest.raises(RuntimeError):
        O.Oracle(feddes_case(feddes=None))
    deep = FEDDES2.copy()
    deep[1, 3] = 2.5   # ZROOT below the 2 m deep bottom nodes
    with pytest.raises(RuntimeError):
        O.Oracle(feddes_case(feddes=deep))
    O.Oracle(feddes_case(feddes=deep, scf=0.0))  # ETRAN not used: accepted


def test_vegetated_ensemble_member_transpires():
    """inputs.with_vegetation on a small ensemble draw: both vegetation
    types present, no sink while it rains, a sink once it evaporates."""
    import oracle as O
    from pycathy_wrapper_gb300.inputs import config2_members, with_vegetation
    c = with_vegetation(config2_members(1, tmax=50000.0, min_cells=8, max_cells=10)[0])
    o = O.Oracle(c)
    assert o.step() == 0
    q, vt = o.qtranie()
    assert set(np.unique(vt)) == {1, 2} and not q.any()
    while o.state()[1] < 45000.0:
        assert o.step() == 0
    q, _ = o.qtranie()
    assert q.min() == 0.0 and q.max() > 0.0


def test_project_reader_parses_feddes_and_root_map():
    case = load_golden_case("weill")
    assert case.soil.scf == 1.0
    assert np.allclose(case.soil.feddes, [[0.0, -4.0, -150.0, 1.0, 1.0, 1.0]])
    assert case.soil.root_map.shape == case.dem.dem.shape
    assert np.all(case.soil.root_map == 1.0)


def test_project_writer_round_trips_feddes(tmp_path):
    from pycathy_wrapper_gb300.project import read_project
    from pycathy_wrapper_gb300.pycathy import write_project
    case = feddes_case()
    write_project(case, str(tmp_path))
    back = read_project(str(tmp_path))
    assert np.allclose(back.soil.feddes, FEDDES2)
    assert np.array_equal(back.soil.root_map, case.soil.root_map)
    assert back.soil.scf == 1.0
