"""C-ABI library: builds, loads, exports every declared symbol; host-side
mesh construction matches the oracle (and so the reference's grid3d); no
CPU fallback when no GPU is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, GOLDEN, has_gpu, load_golden_case


def _declared():
    src = open(os.path.join(ROOT, "include", "cathy_gb300.h")).read()
    return sorted(set(re.findall(r"\b(cathy_gb300_\w+)\s*\(", src)))


def test_exports_every_declared_symbol():
    from pycathy_wrapper_gb300 import _lib
    L = _lib.load()
    names = _declared()
    assert len(names) >= 18
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.EXPORTS, n
    assert L.cathy_gb300_version() >= 100


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_cpu_fallback_without_device():
    from pycathy_wrapper_gb300 import _lib
    from pycathy_wrapper_gb300.api import Simulation
    from pycathy_wrapper_gb300.inputs import config0
    assert _lib.load().cathy_gb300_device_count() == 0
    with pytest.raises(_lib.CathyError) as ei:
        Simulation(config0(tmax=10.0))
    assert ei.value.code == _lib.ENODEV


@pytest.mark.parametrize("key", ["weill", "soil3d"])
def test_host_mesh_matches_oracle(key):
    import oracle as O
    from pycathy_wrapper_gb300.api import build_mesh
    case = load_golden_case(key)
    m = build_mesh(case, iopt=1)
    o = O.Oracle(case)
    om = o.mesh()
    assert (m["n"], m["nt"], m["nnod"], m["ntri"]) == (o.n, o.nt, o.nnod, o.ntri)
    np.testing.assert_array_equal(m["tetra"], om["tetra"])
    np.testing.assert_array_equal(m["x"], om["x"])
    np.testing.assert_array_equal(m["y"], om["y"])
    np.testing.assert_array_equal(m["z"], om["z"])
    # full CSR pattern == symmetric expansion of STRPIC's upper storage
    topol, ja = om["topol"], om["ja"]
    rows = np.repeat(np.arange(o.n), np.diff(topol))
    up = set(zip(rows.tolist(), (ja - 1).tolist()))
    full = up | {(j, i) for i, j in up}
    mrows = np.repeat(np.arange(m["n"]), np.diff(m["rowptr"]))
    got = set(zip(mrows.tolist(), m["cols"].tolist()))
    assert got == full
    assert len(m["cols"]) == 2 * o.nterm - o.n


def test_host_mesh_newton_pattern_matches_strnew():
    import oracle as O
    from pycathy_wrapper_gb300.api import build_mesh
    from pycathy_wrapper_gb300.inputs import config0
    case = config0()
    case.parm.iopt = 2
    m = build_mesh(case, iopt=2)
    o = O.Oracle(case)
    om = o.mesh()
    np.testing.assert_array_equal(m["rowptr"], om["topol"] - 1)
    np.testing.assert_array_equal(m["cols"], om["ja"] - 1)
    np.testing.assert_array_equal(m["tetra"], o.tetra_gen3d())


def test_mesh_with_inactive_cells_and_zones():
    import oracle as O
    from pycathy_wrapper_gb300.api import build_mesh
    from pycathy_wrapper_gb300.inputs import config0
    case = config0()
    dem = case.dem.dem.copy()
    dem[0, 0] = 0.0
    dem[5, 7] = 0.0
    case.dem.dem = dem
    zone = np.ones(dem.shape, np.int32)
    zone[:, 10:] = 2
    case.dem.zone = zone
    from pycathy_wrapper_gb300.inputs import Soil
    case.soil = Soil.homogeneous(case.dem.nstr, nzone=2)
    m = build_mesh(case, iopt=1)
    o = O.Oracle(case)
    om = o.mesh()
    np.testing.assert_array_equal(m["tetra"], om["tetra"])
    np.testing.assert_array_equal(m["z"], om["z"])


def test_gen3d_vertical_modes_and_refusals():
    """IVERT 0, 1, 2 and 4 build the same mesh in the host library and the
    oracle; IVERT 3 (a per-node depth map, gen3d.f:67-68) is refused by
    both instead of being built as another mode."""
    import oracle as O
    from pycathy_wrapper_gb300.api import build_mesh
    from pycathy_wrapper_gb300.inputs import config0
    for ivert in (0, 1, 2, 4):
        case = config0()
        case.dem.ivert = ivert
        m = build_mesh(case, iopt=1)
        np.testing.assert_array_equal(m["z"], O.Oracle(case).mesh()["z"])
    case = config0()
    case.dem.ivert = 3
    with pytest.raises(Exception):
        build_mesh(case, iopt=1)
    with pytest.raises(RuntimeError):
        O.Oracle(case)


def test_bc_lists_held_constant_or_refused(tmp_path):
    """nansfdirbc / nansfneubc: blocks that repeat the first one (or start
    at or after TMAX) are accepted; values that change before TMAX, which
    BCNXT would interpolate, are refused."""
    from pycathy_wrapper_gb300.project import _read_bc_list
    p = tmp_path / "nansfneubc"
    same = "0 time\n0 2 ZERO NQ\n5\n6\n1.0e-6\n2.0e-6\n"
    p.write_text(same + same.replace("0 time", "600 time"))
    ids, vals = _read_bc_list(str(p), tmax=3600.0)
    assert list(ids) == [5, 6] and list(vals) == [1e-6, 2e-6]
    p.write_text(same + same.replace("0 time", "600 time").replace("2.0e-6", "3.0e-6"))
    with pytest.raises(ValueError):
        _read_bc_list(str(p), tmax=3600.0)
    ids, vals = _read_bc_list(str(p), tmax=600.0)  # the change comes at TMAX
    assert list(vals) == [1e-6, 2e-6]
    p.write_text("0 time\n0 0 ZERO NQ\n1800 time\n0 0 ZERO NQ\n")
    assert _read_bc_list(str(p)) is None


def test_reader_refuses_ponded_initial_conditions(tmp_path):
    """IPOND != 0 with ISIMGR = 2 (ponded initial heads, datin.f:380-410)
    needs surface routing: refused; with ISIMGR <= 1 the reference itself
    ignores IPOND (datin.f:381)."""
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.project import read_project
    from pycathy_wrapper_gb300.pycathy import write_project
    case = config0(tmax=600.0)
    for isimgr, ok in ((1, True), (2, False)):
        case.parm.isimgr = isimgr
        prj = tmp_path / f"p{isimgr}"
        write_project(case, str(prj))
        ic = prj / "input" / "ic"
        lines = ic.read_text().splitlines()
        lines[0] = f"{case.bc.indp} 1\tINDP IPOND"
        ic.write_text("\n".join(lines + ["0.05\tPONDNOD"]) + "\n")
        if ok:
            assert read_project(str(prj)).bc.indp == case.bc.indp
        else:
            with pytest.raises(ValueError):
                read_project(str(prj))


def test_variable_relaxation_refused():
    """NLRELX = 2 (RELXOM's per-iteration relaxation factor) is refused by
    the oracle and the reader, as by the engine, rather than run without
    relaxation."""
    import oracle as O
    from pycathy_wrapper_gb300.inputs import config0
    case = config0(tmax=600.0)
    case.parm.nlrelx = 2
    with pytest.raises(RuntimeError):
        O.Oracle(case)
    case.parm.nlrelx = 0
    case.parm.iopt, case.parm.isolv = 2, 1   # a GMRES/TFQMR choice of NSYSLV
    with pytest.raises(RuntimeError):
        O.Oracle(case)
    case.parm.iopt = 1                        # Picard does not read ISOLV
    O.Oracle(case)


def test_reader_refuses_peat_and_nudging(tmp_path):
    """IPEAT = 1 (peat deformation) and NUDN > 0 (nudging observations) are
    refused by the project reader; the zero settings every stored example
    uses read as before."""
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.project import read_project
    from pycathy_wrapper_gb300.pycathy import write_project
    case = config0(tmax=600.0)
    write_project(case, str(tmp_path))
    read_project(str(tmp_path))
    soil = tmp_path / "input" / "soil"
    txt = soil.read_text()
    soil.write_text(txt.replace("0 0.0\tIPEAT SCF", "1 0.0\tIPEAT SCF"))
    with pytest.raises(ValueError):
        read_project(str(tmp_path))
    soil.write_text(txt)
    (tmp_path / "input" / "nudging").write_text("0 2 0\tNUDFLAG NUDN WFLAG\n")
    with pytest.raises(ValueError):
        read_project(str(tmp_path))
    (tmp_path / "input" / "nudging").write_text("0 0 0\tNUDFLAG NUDN WFLAG\n")
    read_project(str(tmp_path))
