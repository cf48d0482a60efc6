"""Drop-in for pyCATHY's processor calls: run CATHY projects on the GPU.

pyCATHY runs a simulation by compiling CATHY and calling ``./cathy`` in the
project directory (pyCATHY/cathy_tools.py:669, ``run_processor``), and runs
a data-assimilation ensemble by calling ``./cathy`` in every member folder
from a process pool (pyCATHY/DA/cathy_DA.py:1389, through
``subprocess_run_multi`` at pyCATHY/cathy_tools.py:76-98).  The functions
here take the same project folders, read the same input files
(:mod:`pycathy_wrapper_gb300.project`), run the subsurface solver on the GPU
-- an ensemble as one batched solve -- and write the output files pyCATHY
reads back: ``output/psi`` (pressure heads, read by
pyCATHY/importers/cathy_outputs.py:480 ``read_psi``), ``output/sw`` (water
saturation, ``read_sw`` at :418), ``output/mbeconv`` (mass balance and
convergence per time step, read by pyCATHY/importers/cathy_outputs.py:607
``read_mbeconv``; row format of cathy_main.f:3269-3273) and
``output/iter`` (the nonlinear-iteration log, conver.f:44-45).
"""
from __future__ import annotations

import os
from typing import List, Sequence

import numpy as np

from .api import Simulation
from .project import read_project


def _fmt_e(v, w, d):
    return f"{v:{w}.{d}E}"


def write_psi(path: str, snapshots) -> None:
    """``snapshots``: iterable of (nstep, time, heads).  Block header as the
    reference's DETOUT writes it, then the heads five per line (E15.6)."""
    with open(path, "w") as f:
        for nstep, time, p in snapshots:
            f.write(f"{int(nstep):7d}{_fmt_e(float(time), 16, 8)}     NSTEP   TIME\n")
            p = np.asarray(p, float)
            for a in range(0, len(p), 5):
                f.write("".join(_fmt_e(v, 15, 6) for v in p[a:a + 5]) + "\n")


def write_sw(path: str, snapshots) -> None:
    """``snapshots``: iterable of (nstep, time, saturation).  The file opens
    with the reference's ``  0   HSPSW`` line (cathy_main.f:2821, format at
    :4134); each block is laid out like ``psi`` (detout.f:44-45), which
    pyCATHY's ``read_sw`` (importers/cathy_outputs.py:418) parses."""
    with open(path, "w") as f:
        f.write("  0   HSPSW\n")
        for nstep, time, sw in snapshots:
            f.write(f"{int(nstep):7d}{_fmt_e(float(time), 16, 8)}     NSTEP   TIME\n")
            sw = np.asarray(sw, float)
            for a in range(0, len(sw), 5):
                f.write("".join(_fmt_e(v, 15, 6) for v in sw[a:a + 5]) + "\n")


def write_iter(path: str, parm, iter_records) -> None:
    """The nonlinear-iteration log: the parameter header of
    cathy_main.f:3960-3972 (written at :2863), a ``(NSTEP: ...)`` line at the
    start of every time-step attempt (format at :3973, written at :2985) and
    one line per Picard/Newton iteration with the convergence and residual
    norms and the heads at IKMAX (conver.f:44-45, format at :103)."""
    with open(path, "w") as f:
        f.write(f"     IOPT   (1 PICARD, 2 NEWTON)             = {int(parm.iopt):6d}\n")
        f.write(f"     NLRELX (0 NORELX,1 CONS RELX,2 VAR RELX)= {int(parm.nlrelx):6d}\n")
        f.write("     KSLOPE (0 ANA, 1 KSL/ANA, 2 KSL/C-DIFF,\n")
        f.write(f"             3 LOC KSL/ANA, 4 LOC TAN-SLOPE) = {int(parm.kslope):6d}\n")
        f.write(f"     TOLUNS (TOLERANCE FOR NONLINEAR ITER)   = {_fmt_e(parm.toluns, 15, 5)}\n")
        f.write(f"     TOLSWI (TOLERANCE FOR BC SWITCHING)     = {_fmt_e(parm.tolswi, 15, 5)}\n")
        f.write(f"     L2NORM (0 INFINITY NORM, ELSE L2 NORM)  = {int(parm.l2norm):6d}\n")
        f.write("\n nlinr  linr converg error norms  node   PNEW at   POLD at   resid error norms\n")
        f.write("  iter  iter       PL2      PINF IKMAX     IKMAX     IKMAX       FL2      FINF\n")
        f.write(" " + "=" * 77 + "\n")
        for r in iter_records:
            if int(r["iter"]) == 1:
                f.write(" " * 23 + f" (NSTEP: {int(r['nstep']):5d}  DELTAT: "
                        f"{_fmt_e(r['deltat'], 12, 4)}  TIME: {_fmt_e(r['time'], 12, 4)})\n")
            f.write(f"{int(r['iter']):6d}{int(r['niter']):6d}{_fmt_e(r['pl2'], 10, 3)}"
                    f"{_fmt_e(r['pinf'], 10, 3)}{int(r['ikmax']):6d}"
                    f"{_fmt_e(r['pnew_ik'], 10, 2)}{_fmt_e(r['pold_ik'], 10, 2)}"
                    f"{_fmt_e(r['fl2'], 10, 3)}{_fmt_e(r['finf'], 10, 3)}\n")


_MBE_HDR = (
    "#NSTEP       DELTAT         TIME  NLIN   AVG.LIN       STORE1       STORE2       DSTORE"
    "   CUM.DSTORE       VIN  CUM.VIN       VOUT    CUM.VOUT   VIN+VOUT   CUM. VIN  M.BAL.ERR"
    "   REL. MBE   CUM. MBE      CUM.\n"
    "#                                 ITER.    ITER.                             (>0 x inc)"
    "                                                                      + VOUT  (Vi+Vo-Ds)"
    "        (%)             ABS(MBE)\n")


def write_mbeconv(path: str, step_records, initial_volume: float) -> None:
    """One row per accepted time step with the 19 columns of the reference's
    mbeconv file."""
    with open(path, "w") as f:
        f.write(f"#INITIAL VOLUME OF WATER IN THE SUBSURFACE = {initial_volume:12.5E}\n")
        f.write(_MBE_HDR)
        for r in step_records:
            it = max(int(r["iter"]), 1)
            vals = [
                f"{int(r['nstep']):6d}", _fmt_e(r["deltat"], 12, 6), _fmt_e(r["time"], 12, 6),
                f"{it:5d}", _fmt_e(r["nitert"] / it, 9, 3), _fmt_e(r["store1"], 12, 6),
                _fmt_e(r["store2"], 12, 6), _fmt_e(r["dstore"], 12, 5),
                _fmt_e(r["cdstor"], 12, 5), _fmt_e(r["vin"], 9, 3), _fmt_e(r["cvin"], 9, 3),
                _fmt_e(r["vout"], 10, 3), _fmt_e(r["cvout"], 10, 3),
                _fmt_e(r["vin"] + r["vout"], 10, 3), _fmt_e(r["cvin"] + r["cvout"], 10, 3),
                _fmt_e(r["erras"], 10, 3), _fmt_e(r["errel"], 10, 3), _fmt_e(r["cerras"], 10, 3),
                _fmt_e(r["caeras"], 9, 3)]
            f.write(" ".join(vals) + "\n")


def _write_member(prj: str, parm, p0, sw0, result, sw, its, recs) -> None:
    out = os.path.join(prj, "output")
    os.makedirs(out, exist_ok=True)
    p, t, dt, status = result
    nstep = recs[-1]["nstep"] if recs else 0
    write_psi(os.path.join(out, "psi"), [(0, 0.0, p0), (nstep, t, p)])
    write_sw(os.path.join(out, "sw"), [(0, 0.0, sw0), (nstep, t, sw)])
    v0 = (recs[0]["store2"] - recs[0]["cdstor"]) if recs else 0.0
    write_mbeconv(os.path.join(out, "mbeconv"), recs, v0)
    write_iter(os.path.join(out, "iter"), parm, its)


def run_project(prj: str, precision: int = 1, device: int = 0, write: bool = True) -> dict:
    """Run one pyCATHY project folder to TMAX on the GPU (the replacement
    of ``subprocess.run(["./cathy"])``).  Returns heads, time and status."""
    return run_ensemble([prj], precision=precision, device=device, write=write)[0]


def run_ensemble(member_dirs: Sequence[str], precision: int = 1, device: int = 0,
                 write: bool = True) -> List[dict]:
    """Run every member folder of a DA ensemble as ONE batched GPU solve
    (the replacement of the process pool over ``./cathy``).  Members may
    differ in mesh, soil, forcing and initial state; they must share IOPT,
    LUMP and the Picard preconditioner."""
    cases = [read_project(d) for d in member_dirs]
    for c in cases:
        if c.parm.iopt == 1 and c.parm.precond == 0 and precision == 1:
            c.parm.precond = 2  # FP32 batched path: column-line preconditioner
    out = []
    with Simulation(cases, precision=precision, device=device) as s:
        p0 = [s.state(m)[0].copy() for m in range(len(cases))]
        sw0 = [s.saturation(m) for m in range(len(cases))]
        s.run()
        for m, d in enumerate(member_dirs):
            res = s.state(m)
            its, recs = s.records(m)
            if write:
                _write_member(d, cases[m].parm, p0[m], sw0[m], res, s.saturation(m), its, recs)
            out.append(dict(dir=d, pnew=res[0], time=res[1], deltat=res[2],
                            status=int(res[3]), steps=len(recs)))
    return out


# ---------------------------------------------------------------------------
# project writer (the files pyCATHY's update_* methods write)
# ---------------------------------------------------------------------------
def _raster(path, a, west=0.0, south=0.0, dx=1.0, dy=1.0):
    nrow, ncol = a.shape
    with open(path, "w") as f:
        f.write(f"north:     {south + nrow * dy}\nsouth:     {south}\n")
        f.write(f"east:      {west + ncol * dx}\nwest:      {west}\n")
        f.write(f"rows:     {nrow}\ncols:     {ncol}\n")
        for r in a:
            f.write("".join(f"{v:26.17E}" for v in r) + "\n")


def write_project(case, prj: str) -> None:
    """Write a Case as a CATHY project folder (input/parm, input/soil,
    input/dem_parameters, input/ic, input/atmbc, prepro/dem, prepro/zone and
    the Dirichlet/Neumann lists), in the layouts that CATHY's datin.f reads
    and :func:`pycathy_wrapper_gb300.project.read_project` parses."""
    d, s, p, b = case.dem, case.soil, case.parm, case.bc
    inp, pre = os.path.join(prj, "input"), os.path.join(prj, "prepro")
    os.makedirs(inp, exist_ok=True)
    os.makedirs(pre, exist_ok=True)
    with open(os.path.join(inp, "parm"), "w") as f:
        f.write("2 0 0\tIPRT1 NCOUT TRAFLAG\n")
        f.write(f"{p.isimgr} {p.pondh_min!r} 0\tISIMGR PONDH_MIN VELREC\n")
        f.write(f"{p.kslope} {p.tolksl!r}\tKSLOPE TOLKSL\n")
        f.write("-3.0 -1.0 -3.0 -1.0\tPKRL PKRR PSEL PSER\n")
        f.write("-3.0 -2.5 -1.5 -1.0\tPDSE1L PDSE1R PDSE2L PDSE2R\n")
        f.write("0 0 0\tISFONE ISFCVG DUPUIT\n")
        f.write(f"{p.tetaf!r} {p.lump} {p.iopt}\tTETAF LUMP IOPT\n")
        f.write(f"{p.nlrelx} {p.omega!r}\tNLRELX OMEGA\n")
        f.write(f"{p.l2norm} {p.toluns!r} {p.tolswi!r} {p.ernlmx!r}\tL2NORM TOLUNS TOLSWI ERNLMX\n")
        f.write(f"{p.ituns} {p.ituns1} {p.ituns2}\tITUNS ITUNS1 ITUNS2\n")
        f.write(f"{p.isolv} {p.itmxcg} {p.tolcg!r}\tISOLV ITMXCG TOLCG\n")
        f.write(f"{p.deltat!r} {p.dtmin!r} {p.dtmax!r} {p.tmax!r}\tDELTAT DTMIN DTMAX TMAX\n")
        f.write(f"{p.dtmaga!r} {p.dtmagm!r} {p.dtreds!r} {p.dtredm!r}\tDTMAGA DTMAGM DTREDS DTREDM\n")
        f.write(f"4 2 1 {p.tmax!r}\tIPRT VTKF NPRT (TIMPRT(I),I=1,NPRT)\n")
        f.write("1 1\tNUMVP (NODVP(I),I=1,NUMVP)\n0\tNR\n0\tNUM_QOUT\n1\t(ID_QOUT(I),I=1,NUM_QOUT)\n")
    nzone, nstr = s.nzone, d.nstr
    with open(os.path.join(inp, "dem_parameters"), "w") as f:
        f.write(f"{d.delta_x!r}\n{d.delta_y!r}\n{d.factor!r}\n1\n{nzone}\t{nstr}\t25\n")
        f.write(f"{d.ivert}\t1\t{d.base!r}\n")
        f.write("\t".join(repr(float(z)) for z in d.zratio) + "\n")
    with open(os.path.join(inp, "soil"), "w") as f:
        f.write(f"{s.pmin!r}\tPMIN\n0 {s.scf!r}\tIPEAT SCF\n0.4 0.225\tCBETA0,CANG\n")
        f.write("0.0 -4.0 -150.0 1.0 1.0 1.0\tPCANA,PCREF,PCWLT,ZROOT,PZ,OMGC\n")
        f.write("0\tIVGHU\n0.02 2 2 0 0.333\tHUALFA,HUBETA,HUGAMA,HUPSIA,HUSWR\n1\tHUN\n")
        f.write("-5 1\tHUA,HUB\n1.2 0 -0.345\tBCBETA,BCRMC,BCPSAT\n")
        keys = ("permx", "permy", "permz", "elstor", "poros", "vgn", "vgrmc", "vgpsat")
        for layer in range(nstr):
            for z in range(nzone):
                f.write(" ".join(repr(float(getattr(s, k)[z, layer])) for k in keys) + "\n")
    with open(os.path.join(inp, "ic"), "w") as f:
        f.write(f"{b.indp} 0\tINDP IPOND\n")
        if b.indp in (3, 4):
            f.write(f"{b.wtposition!r}\tWTPOSITION\n")
        elif b.indp == 0:
            f.write(f"{float(np.ravel(b.pinit)[0])!r}\tPCONST\n")
        elif b.indp == 1:
            pv = np.ravel(b.pinit)
            for a in range(0, len(pv), 5):
                f.write(" ".join(repr(float(v)) for v in pv[a:a + 5]) + "\n")
    with open(os.path.join(inp, "atmbc"), "w") as f:
        f.write(f"{b.hspatm} {b.ieto}\tHSPATM IETO\n")
        for k, t in enumerate(np.ravel(b.atmtim)):
            f.write(f"{float(t)!r}\tTIMEIN\n")
            v = np.atleast_1d(b.atminp[k])
            f.write(" ".join(repr(float(x)) for x in v) + "\tATMINP\n")
    for name, ids, vals in (("nansfdirbc", b.contp, b.presc), ("nansfneubc", b.contq, b.q)):
        with open(os.path.join(inp, name), "w") as f:
            ids = np.zeros(0, np.int32) if ids is None else np.ravel(ids)
            vals = np.zeros(0) if vals is None else np.ravel(vals)
            f.write("0.0\tTIME\n")
            f.write(f"0 {len(ids)}\tNDIR NDIRC\n")
            for a in ids:
                f.write(f"{int(a)}\n")
            for v in vals:
                f.write(f"{float(v)!r}\n")
    _raster(os.path.join(pre, "dem"), np.asarray(d.dem, float), d.west, d.south,
            d.delta_x, d.delta_y)
    if d.zone is not None:
        _raster(os.path.join(pre, "zone"), np.asarray(d.zone, float), d.west, d.south,
                d.delta_x, d.delta_y)
