"""Generate the golden fixtures from the reference's stored CATHY runs.

The ETRAN record of the first time step (the first line of the run's
fort.666: TIME and QTRAN, the sum of QTRANIE) is kept as well.

Run where the reference checkout is available, giving its path:

    python tests/golden/make_golden.py <path to the reference checkout>

For each example project it stores (a) the project inputs as parsed by
``pycathy_wrapper_gb300.project.read_project`` and (b) the values the
reference CATHY binary printed for that project: the GEN3D mesh
(``output/grid3d``), NTERM (``output/risul``), and the first nonlinear
iteration record of the first time step (``output/iter`` and the linear
solver line of ``output/risul``).  The first iteration is a clean known
answer for initial conditions + assembly + boundary conditions + IC(0)-PCG:
surface routing only starts once ponding occurs (cathy_main.f:2993).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from pycathy_wrapper_gb300.project import read_project  # noqa: E402

EXAMPLES = {
    "weill": "examples/SSHydro/weill_exemple",
    "soil3d": "examples/SSHydro/soil3d_from_weill",
    # spatially variable evaporation with SCF = 1 over a DEM with no-data
    # cells: the only forcing of its first iteration is the Feddes sink
    "etp": "examples/SSHydro/atmbc_spatially_from_weill_withnodata",
    # a 1,271-node catchment forced by an Earth-observation ET/rain series
    # (30 spatial records): it never ponds, so its whole 29-day run is a
    # subsurface run -- every iter record and mbeconv row is kept
    "eo": "examples/EOdata/mapping_atmbc_from_EO_dataset",
    # the same catchment with the coarse EO series: 6,069 stored steps
    "eoc": "examples/EOdata/mapping_atmbc_from_coarse_EO_dataset",
    # a DA ensemble member started from nodal heads (INDP = 1); its risul
    # keeps no solver lines.  (Member 1's stored iter is the same file
    # while its ic was rewritten by the analysis step: not a pin.)
    "da2": "examples/DA/DA_with_swc/DA_SMC/DA_Ensemble/cathy_2",
}
# keys whose whole run is kept: every record of output/iter and
# output/mbeconv (as printed)
WHOLE_RUN = {"eo", "eoc"}


def run_records(prj):
    """Every nonlinear-iteration record of output/iter (the step header's
    NSTEP and DELTAT, then ITER, NITER, PL2, PINF, IKMAX) and every row of
    output/mbeconv (19 columns, as printed)."""
    import re
    it = []
    head = None
    for ln in open(os.path.join(prj, "output", "iter")):
        m = re.search(r"NSTEP:\s+(\d+)\s+DELTAT:\s+([^\s)]+)", ln)
        if m:
            head = (int(m.group(1)), float(m.group(2)))
            continue
        t = ln.split()
        if head and len(t) == 9 and t[0].isdigit():
            it.append((head[0], int(t[0]), int(t[1]), int(t[4]), head[1], float(t[2]),
                       float(t[3])))
    mb = []
    for ln in open(os.path.join(prj, "output", "mbeconv")):
        if ln.startswith("#") or not ln.strip():
            continue
        try:
            mb.append([float(x) for x in ln.split()])
        except ValueError:
            pass
    it = np.array(it)
    return dict(it_int=it[:, :4].astype(np.int32), it_dt=it[:, 4], it_norm=it[:, 5:7],
                mbeconv=np.array(mb))


def first_iter(prj):
    rec = None
    for ln in open(os.path.join(prj, "output", "iter")):
        t = ln.split()
        if len(t) == 9 and t[0] == "1":
            rec = dict(iter=int(t[0]), niter=int(t[1]), pl2=float(t[2]),
                       pinf=float(t[3]), ikmax=int(t[4]), pnew_ik=float(t[5]),
                       pold_ik=float(t[6]), fl2=float(t[7]), finf=float(t[8]))
            break
    nterm = None
    lin = None
    risul = os.path.join(prj, "output", "risul")
    for ln in (open(risul) if os.path.exists(risul) else []):
        if "NTERM" in ln and nterm is None:
            nterm = int(ln.split("=")[1])
        if "<<SYMMETRIC SOLVER>>" in ln and lin is None:
            t = ln.split()
            lin = dict(niter=int(t[0]), err=float(t[1]), res=float(t[2]))
    return rec, nterm, lin


def case_to_npz(case, path):
    """The parsed inputs of a project as arrays (+ a JSON of the scalars)."""
    d, s, p, b = case.dem, case.soil, case.parm, case.bc
    arrs = dict(dem=d.dem, zratio=d.zratio,
                zone=d.zone if d.zone is not None else np.ones_like(d.dem, np.int32))
    for k in ("permx", "permy", "permz", "elstor", "poros", "vgn", "vgrmc", "vgpsat"):
        arrs["soil_" + k] = getattr(s, k)
    if s.feddes is not None:
        arrs["soil_feddes"] = np.asarray(s.feddes, float)
    if s.root_map is not None:
        arrs["soil_root_map"] = np.asarray(s.root_map, float)
    arrs["atmtim"] = b.atmtim
    arrs["atminp"] = b.atminp
    if b.pinit is not None:
        arrs["pinit"] = np.asarray(b.pinit, float)
    meta = dict(delta_x=d.delta_x, delta_y=d.delta_y, base=d.base, ivert=d.ivert,
                west=d.west, south=d.south, factor=d.factor,
                pmin=s.pmin, scf=s.scf, kslope=s.kslope, tolksl=s.tolksl,
                parm={k: getattr(p, k) for k in p.__dataclass_fields__},
                hspatm=b.hspatm, ieto=b.ieto, indp=b.indp, wtposition=b.wtposition)
    np.savez_compressed(path, meta=json.dumps(meta), **arrs)


def main(ref):
    out = {}
    for key, rel in EXAMPLES.items():
        prj = os.path.join(ref, rel)
        case = read_project(prj)
        case_to_npz(case, os.path.join(HERE, f"{key}_case.npz"))
        if key in WHOLE_RUN:
            np.savez_compressed(os.path.join(HERE, f"{key}_run.npz"), **run_records(prj))
        if key == "etp":
            # the mesh of a DEM with no-data cells, as GEN3D wrote it
            np.savez_compressed(os.path.join(HERE, "etp_xyz.npz"), xyz=np.array(
                open(os.path.join(prj, "output", "xyz")).read().splitlines()))
        if key == "eo":
            # the binary's own text of its first 200 steps: mbeconv's three
            # header lines and 200 rows, the first 700 lines of iter, the
            # header line and 200 rows of wtdepth and hgsfdet, and psi's
            # second block (the heads after step 1)
            rd = lambda f: open(os.path.join(prj, "output", f)).read().splitlines()
            psi = rd("psi")
            blk = [i for i, ln in enumerate(psi) if ln.endswith("NSTEP   TIME")]
            np.savez_compressed(os.path.join(HERE, "eo_text.npz"),
                                mbeconv_head=np.array(rd("mbeconv")[:203]),
                                iter_head=np.array(rd("iter")[:700]),
                                wtdepth_head=np.array(rd("wtdepth")[:201]),
                                hgsfdet_head=np.array(rd("hgsfdet")[:201]),
                                psi_step1=np.array(psi[blk[1]:(blk + [len(psi)])[2]]),
                                sw_all=np.array(rd("sw")),
                                cumflowvol_head=np.array(rd("cumflowvol")[:202]))
        rec, nterm, lin = first_iter(prj)
        out[key] = dict(source=rel, first_iter=rec, nterm=nterm, linear=lin)
        # ETRAN's record of the first time step (cathy_main.f:2929-2940
        # writes TIME, QTRAN = sum of QTRANIE, RWU to unit 666)
        f666 = os.path.join(prj, "fort.666")
        if os.path.exists(f666):
            t0, q0 = (float(v) for v in open(f666).readline().split()[:2])
            out[key]["etran_first"] = dict(time=t0, qtran=q0)
        if key == "weill":
            g = open(os.path.join(prj, "output", "grid3d")).read().split("\n")
            nnod, n, nt = (int(v) for v in g[0].split())
            tet = np.array(" ".join(g[1:1 + nt]).split(), np.int32).reshape(nt, 5)
            xyz = np.array(" ".join(g[1 + nt:1 + nt + n]).split(), float).reshape(n, 3)
            np.savez_compressed(os.path.join(HERE, "weill_grid3d.npz"), tetra=tet,
                                xyz=xyz, nnod=nnod)
            out[key]["grid3d"] = dict(nnod=nnod, n=n, nt=nt)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
