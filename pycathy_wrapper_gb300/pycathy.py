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
import time
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


def write_grid3d(path: str, mesh) -> None:
    """The 3-D mesh as GEN3D writes it for IPRT1 = 3 (gen3d.f:96-102,
    formats 1030-1050): NNOD N NT, the NT tetrahedra (4 nodes + material, in
    GEN3D's node order: the mesh of :func:`mesh_gen3d`), the N node
    coordinates; pyCATHY's ``read_grid3d`` (importers/cathy_outputs.py:15)
    parses it."""
    x, y, z, tetra = mesh["x"], mesh["y"], mesh["z"], np.asarray(mesh["tetra"])
    with open(path, "w") as f:
        f.write(f"{int(mesh['nnod']):9d}{len(x):9d}{len(tetra):9d}\n")
        for t in tetra:
            f.write("".join(f"{int(v):7d}" for v in t[:5]) + "\n")
        for a, b, c in zip(x, y, z):
            f.write(_fmt_e(a, 15, 6) + _fmt_e(b, 15, 6) + _fmt_e(c, 15, 6) + "\n")


def write_xyz(path: str, mesh) -> None:
    """Node coordinates as GEN3D writes them for IPRT1 = 3 (gen3d.f:92-95,
    formats 1010-1020); pyCATHY's ``read_xyz`` (:177) parses it."""
    x, y, z = mesh["x"], mesh["y"], mesh["z"]
    with open(path, "w") as f:
        f.write(f"{int(mesh['nnod']):7d}{len(x):7d}  NNOD   N\n")
        for i, (a, b, c) in enumerate(zip(x, y, z)):
            f.write(f"{i + 1:7d}" + _fmt_e(a, 15, 6) + _fmt_e(b, 15, 6) + _fmt_e(c, 15, 6) + "\n")


def water_table(p, z, nnod: int, nstr: int, nodvp) -> List[float]:
    """Water-table elevation at the NODVP columns (wtdepth.f:18-46): from
    the bottom layer up, the first pair of a saturated node below an
    unsaturated one, interpolated linearly in the head; with no such pair,
    the ponded surface level if the surface node is saturated, else the
    bottom of the column.  Node k*nnod + c is column c, layer k (0 = top)."""
    out = []
    for nv in nodvp:
        c = int(nv) - 1
        wt, flag = z[c], 0
        for j in range(nstr, 0, -1):
            i1, i2 = c + j * nnod, c + (j - 1) * nnod
            if p[i1] >= 0.0 and p[i2] < 0.0 and flag == 0:
                rc = (z[i1] - z[i2]) / (p[i1] - p[i2])
                wt, flag = z[i1] - rc * p[i1], 1
            elif p[i1] >= 0.0 and p[i2] < 0.0 and flag == 1:
                flag = 2
            elif j == 1 and p[i2] >= 0.0 and flag == 0:
                wt, flag = z[c] + p[i2], 3
            elif j == 1 and flag == 0:
                wt, flag = z[c + nstr * nnod], 4
        out.append(float(wt))
    return out


def write_wtdepth(path: str, rows) -> None:
    """``rows``: (time, [water table at each NODVP column]) per accepted
    step; header of cathy_main.f:2872 (format :4042), rows in format 1020
    of wtdepth.f (70 values of 1PE15.6 per line)."""
    with open(path, "w") as f:
        f.write("#TIME      <--- WTDEPTH(NODVP(I)), I=1,2,...,NUMVP --->\n")
        for t, wt in rows:
            vals = [float(t)] + [float(w) for w in wt]
            for a in range(0, len(vals), 70):
                f.write("".join(_fmt_e(v, 15, 6) for v in vals[a:a + 70]) + "\n")


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
        f.write(f"#INITIAL VOLUME OF WATER IN THE SUBSURFACE = {initial_volume:13.5E}\n")
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


def write_hgsfdet(path: str, step_records) -> None:
    """The seepage-face hydrograph (hgsfdet: header mbinit.f:30, rows
    cathy_main.f:3666, format I7,4(4X,1PE17.9)): per accepted step NSTEP,
    DELTAT, TIME, the seepage-face volume VSFFLW = (SFFLW + SFFLWP) DELTAT/2
    (masbal.f) and VSFFLW/DELTAT.  The reference writes it whether or not
    the project has seepage faces."""
    with open(path, "w") as f:
        f.write("# NSTEP            DELTAT              TIME"
                "  NET SEEPFACE VOL  NET SEEPFACE FLX\n")
        prev = 0.0
        for r in step_records:
            dt = r["deltat"]
            sf = r.get("sfflw", 0.0)
            vol = (sf + prev) * (0.5 * dt if dt < 1.0e15 else 1.0)
            prev = sf
            f.write(f"{int(r['nstep']):7d}" + "".join(
                f"    {v:17.9E}" for v in (dt, r["time"], vol, vol / dt)) + "\n")


def write_cumflowvol(path: str, step_records) -> None:
    """Cumulative flow volumes (cumflowvol: header mbinit.f:95-97, rows
    cathy_main.f:3677 in format I7,6(1PE10.2),1PE12.4): per accepted step
    NSTEP, DELTAT, TIME and the running sums VSFTOT (seepage faces, the
    trapezoids of SFFLW), VNDTOT and VNNTOT (non-atmospheric Dirichlet and
    Neumann nodes), VNUDTOT (nudging, 0 here) and VTOT (VIN + VOUT)
    (cathy_main.f:3259-3263)."""
    with open(path, "w") as f:
        f.write(" " * 21 + "#***** Cumulative flow volumes ***** \n")
        f.write("# Nstep    Deltat      Time  SeepageF  nansfDir  nansfNeu   Nudging"
                "  net (VTOT)\n")
        vsf = vnd = vnn = vtot = 0.0
        prev = 0.0
        for r in step_records:
            dt = r["deltat"]
            sf = r.get("sfflw", 0.0)
            vsf += (sf + prev) * (0.5 * dt if dt < 1.0e15 else 1.0)
            prev = sf
            vnd += r.get("vnd", 0.0)
            vnn += r.get("vnn", 0.0)
            vtot += r["vin"] + r["vout"]
            f.write(f"{int(r['nstep']):7d}" + "".join(
                _fmt_e(v, 10, 2) for v in (dt, r["time"], vsf, vnd, vnn, 0.0)) +
                _fmt_e(vtot, 12, 4) + "\n")


_PHASE_LINES = (
    " TOT CPU FOR UNSAT CHARACTERISTICS    = ", " TOT CPU FOR INIT. OF SYSTEM MATRICES = ",
    " TOT CPU FOR LOCAL SYSTEM ASSEMBLY    = ", " TOT CPU FOR RHS CALCULATION W/O BC'S = ",
    " TOT CPU FOR GLOBAL LHS SYSTEM MATRIX = ", " TOT CPU FOR BC CONTRIBUTIONS TO RHS  = ",
    " TOT CPU FOR LINEAR SOLVER & RESIDUAL = ", " TOT CPU FOR DIR. RESETTING AND DIFMAX= ",
    " TOT CPU FOR B-FLX, M-BAL, SW, & EX-PT= ")


def write_risul(path: str, step_records, iter_records, phase_s, total_s) -> None:
    """The closing summary of the reference's ``risul`` file
    (cathy_main.f:3880-3950, formats 1215, 1400, 1420, 1440, 1450): the
    cumulative mass-balance error, the back-step and linear-failure counts,
    the time spent per phase (here GPU seconds of the nonlinear iterations,
    in the reference's nine CPUVEC buckets, picard.f:66-202; ``phase_s``
    holds them in that order) and the time-step statistics (DTSTAT,
    dtstat.f:8-24)."""
    recs, its = list(step_records), list(iter_records)
    total = max(float(total_s), 1e-30)
    nl = sum(phase_s)
    with open(path, "w") as f:
        if recs:
            r = recs[-1]
            vtot = r["cvin"] + r["cvout"]
            if vtot != 0.0:
                f.write(f"\n  CUMULATIVE (TOTAL) MBE BASED ON CERRAS         : {r['cerras']:12.5E}\n")
                f.write(f"  CUMULATIVE (TOTAL) RELATIVE MBE BASED ON CERRAS: "
                        f"{100.0 * r['cerras'] / vtot:12.5E} %\n")
        nback = sum(int(r["nback"]) for r in recs)
        f.write(f"\n  TOTAL NUMBER OF BACK-STEPPING OCCURRENCES      : {nback:6d}\n")
        f.write("  TOTAL NUMBER OF LINEAR SOLVER FAILURES         :      0\n\n")
        f.write(f"\n  TOT CPU FOR THE SIMULATION           = {total:15.2f} SECONDS  {100.0:6.2f} %\n")
        f.write(f"  TOT CPU FOR NONLINEAR SCHEME         = {nl:15.2f} SECONDS  "
                f"{100.0 * nl / total:6.2f} %\n")
        f.write(f"  TOT CPU FOR OVERHEAD (SEE CODE DESC.)= {total - nl:15.2f} SECONDS  "
                f"{100.0 * (total - nl) / total:6.2f} %\n\n")
        for name, v in zip(_PHASE_LINES, phase_s):
            f.write(f" {name}{v:15.2f} SECONDS  {100.0 * v / total:6.2f} %\n")
        f.write(" " * 41 + "-----------" + " " * 9 + "-------\n")
        f.write(" " * 41 + f"{nl:11.2f} SECONDS  {100.0 * nl / total:6.2f} %\n\n")
        ns = len(recs)
        dts = [r["deltat"] for r in recs]
        ksm = int(np.argmin(dts)) if dts else 0
        kbg = int(np.argmax(dts)) if dts else 0
        nli = len(its)
        lin = sum(int(r["niter"]) for r in its)
        per = lambda a, b: a / b if b else 0.0
        f.write(f"  TOTAL NUMBER OF TIME STEPS           = {ns:8d}\n")
        if dts:
            f.write(f"  SMALLEST TIME STEP SIZE              = {dts[ksm]:11.3E}  AT TIME "
                    f"{recs[ksm]['time']:11.3E}\n")
            f.write(f"  LARGEST  TIME STEP SIZE              = {dts[kbg]:11.3E}  AT TIME "
                    f"{recs[kbg]['time']:11.3E}\n")
            f.write(f"  AVERAGE  TIME STEP SIZE              = {sum(dts) / ns:11.3E}\n")
        f.write(f"  TOTAL NUMBER OF NONLINEAR ITERATIONS = {nli:8d}\n")
        f.write(f"  TOTAL NUMBER OF LINEAR ITERATIONS    = {lin:8d}  (= 0 FOR NONSYM)\n")
        f.write(f"  AVG NL ITERATIONS PER TIME STEP      = {per(nli, ns):8.2f}\n")
        f.write(f"  AVG LINEAR ITERATIONS PER TIME STEP  = {per(lin, ns):8.2f}\n")
        f.write(f"  AVG LIN ITERATIONS PER NL ITERATION  = {per(lin, nli):8.2f}\n")
        f.write(f"  AVG TOT CPU PER TIME STEP            = {per(total, ns):8.2f} SECONDS\n")
        f.write(f"  AVG TOT CPU PER NL ITERATION         = {per(total, nli):8.2f} SECONDS\n")
        f.write(f"  AVG TOT NL CPU PER TIME STEP         = {per(nl, ns):8.2f} SECONDS\n")
        f.write(f"  AVG TOT NL CPU PER NL ITERATION      = {per(nl, nli):8.2f} SECONDS\n")


def drive_outputs(sim, n: int, parms, meshes):
    """Run every member to the end one accepted step at a time (``sim.step``
    advances each running member by exactly one step, so the members'
    trajectories are those of an uninterrupted run) and collect what the
    reference writes along the way: detailed output (heads and saturation)
    at TIME = 0 and at the first step reaching each TIMPRT
    (cathy_main.f:3715-3738), and the water table at the NODVP columns after
    every step (cathy_main.f:3628).  ``sim`` needs step(), state(m),
    saturation(m) and num_steps(m)."""
    snaps = [[(0, 0.0, sim.state(m)[0].copy(), sim.saturation(m))] for m in range(n)]
    kprt, seen = [0] * n, [0] * n
    wt = [[] for _ in range(n)]
    while True:
        nact = sim.step()
        for m in range(n):
            k = sim.num_steps(m)
            if k == seen[m]:
                continue
            seen[m] = k
            p, t = sim.state(m)[:2]
            msh, parm = meshes[m], parms[m]
            if parm.nodvp:
                wt[m].append((t, water_table(p, msh["z"], msh["nnod"], msh["nstr"], parm.nodvp)))
            if kprt[m] < len(parm.timprt) and t >= parm.timprt[kprt[m]]:
                snaps[m].append((k, t, p.copy(), sim.saturation(m)))
                kprt[m] += 1
        if nact == 0:
            break
    for m in range(n):
        k = sim.num_steps(m)
        p, t = sim.state(m)[:2]
        if snaps[m][-1][0] != k:  # the end of the run (TIME = TMAX)
            snaps[m].append((k, t, p.copy(), sim.saturation(m)))
    return snaps, wt


def _write_member(prj: str, parm, mesh, snaps, wt, its, recs, phase_s=None,
                  total_s=0.0) -> None:
    out = os.path.join(prj, "output")
    os.makedirs(out, exist_ok=True)
    write_psi(os.path.join(out, "psi"), [(k, t, p) for k, t, p, _ in snaps])
    write_sw(os.path.join(out, "sw"), [(k, t, sw) for k, t, _, sw in snaps])
    v0 = (recs[0]["store2"] - recs[0]["cdstor"]) if recs else 0.0
    write_mbeconv(os.path.join(out, "mbeconv"), recs, v0)
    write_iter(os.path.join(out, "iter"), parm, its)
    write_hgsfdet(os.path.join(out, "hgsfdet"), recs)
    write_cumflowvol(os.path.join(out, "cumflowvol"), recs)
    if parm.nodvp:
        write_wtdepth(os.path.join(out, "wtdepth"), wt)
    write_grid3d(os.path.join(out, "grid3d"), mesh)
    write_xyz(os.path.join(out, "xyz"), mesh)
    if phase_s is not None:
        write_risul(os.path.join(out, "risul"), recs, its, phase_s, total_s)


def mesh_gen3d(case) -> dict:
    """The host mesh with the tetrahedra in GEN3D's node order (the Picard
    pattern builder sorts each tetrahedron's nodes after GEN3D has written
    grid3d; the Newton mesh keeps GEN3D's order)."""
    from .api import build_mesh
    mesh = build_mesh(case, iopt=2)
    mesh["nstr"] = case.dem.nstr
    return mesh


def write_mesh(prj: str) -> dict:
    """The IPRT1 = 3 run of the reference (gen3d.f:89-111: write the mesh
    and stop), on the host mesh builder: ``output/grid3d`` and
    ``output/xyz``.  pyCATHY runs it to get the mesh
    (pyCATHY/cathy_tools.py:729)."""
    case = read_project(prj)
    mesh = mesh_gen3d(case)
    out = os.path.join(prj, "output")
    os.makedirs(out, exist_ok=True)
    write_grid3d(os.path.join(out, "grid3d"), mesh)
    write_xyz(os.path.join(out, "xyz"), mesh)
    return mesh


def run_project(prj: str, precision: int = 1, device: int = 0, write: bool = True) -> dict:
    """Run one pyCATHY project folder to TMAX on the GPU (the replacement
    of ``subprocess.run(["./cathy"])``; with IPRT1 = 3 in ``input/parm`` it
    writes the mesh files and stops, as the reference does).  Returns heads,
    time and status."""
    if read_project(prj).parm.iprt1 == 3:
        mesh = write_mesh(prj)
        return dict(dir=prj, mesh=mesh, status=1, steps=0)
    return run_ensemble([prj], precision=precision, device=device, write=write)[0]


class _Stepper:
    """The engine seen through the calls of :func:`drive_outputs`."""

    def __init__(self, sim):
        self.sim = sim

    def step(self):
        return self.sim.step()

    def state(self, m):
        return self.sim.state(m)

    def saturation(self, m):
        return self.sim.saturation(m)

    def num_steps(self, m):
        return self.sim.num_records(m)[1]


def run_ensemble(member_dirs: Sequence[str], precision: int = 1, device: int = 0,
                 write: bool = True, rank: int = 0, world: int = 1) -> List[dict]:
    """Run every member folder of a DA ensemble as ONE batched GPU solve
    (the replacement of the process pool over ``./cathy``).  Members may
    differ in mesh, soil, forcing and initial state; they must share IOPT,
    LUMP and the Picard preconditioner.  With ``write`` the members step
    together one accepted step at a time so that the detailed output and
    the water table are taken where the reference takes them; without it
    they run straight to the end.  (The FP32 dot products of the batched
    SpMV are grouped over the members that are active at the time, so the
    two schedules agree to the FP32 rounding of those sums, not bit for
    bit.)

    With ``world`` > 1 the call runs only rank ``rank``'s shard of the
    members (one process per GPU; shards balanced by mesh size, see
    :mod:`pycathy_wrapper_gb300.shard`) and returns that shard's results."""
    if world > 1:
        from .shard import member_nodes, shard_of
        allc = [read_project(d) for d in member_dirs]
        mine = shard_of(member_nodes(allc), rank, world)
        member_dirs = [member_dirs[m] for m in mine]
    cases = [read_project(d) for d in member_dirs]
    for c in cases:
        if c.parm.iopt == 1 and c.parm.precond == 0 and precision == 1:
            c.parm.precond = 2  # FP32 batched path: column-line preconditioner
    out = []
    with Simulation(cases, precision=precision, device=device) as s:
        if write:
            # the phase table of risul needs per-phase timing (kernel by
            # kernel, CUDA events between the phases)
            s.phase_timers(1)
            t0 = time.perf_counter()
            meshes = [mesh_gen3d(c) for c in cases]
            snaps, wt = drive_outputs(_Stepper(s), len(cases), [c.parm for c in cases], meshes)
            total = time.perf_counter() - t0
            ph = [v / 1000.0 for v in s.phase_timers(0).values()]
            # a batch shares the phase times: each member's share is its
            # rows' share of the batch
            rows = np.array([float(sz["n"]) for sz in s.sizes])
            share = rows / rows.sum()
        else:
            s.run()
        for m, d in enumerate(member_dirs):
            res = s.state(m)
            its, recs = s.records(m)
            if write:
                _write_member(d, cases[m].parm, meshes[m], snaps[m], wt[m], its, recs,
                              [v * share[m] for v in ph], total * share[m])
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
        f.write(f"{p.iprt1} 0 0\tIPRT1 NCOUT TRAFLAG\n")
        f.write(f"{p.isimgr} {p.pondh_min!r} 0\tISIMGR PONDH_MIN VELREC\n")
        f.write(f"{p.kslope} {p.tolksl!r}\tKSLOPE TOLKSL\n")
        f.write("-3.0 -1.0 -3.0 -1.0\tPKRL PKRR PSEL PSER\n")
        f.write("-3.0 -2.5 -1.5 -1.0\tPDSE1L PDSE1R PDSE2L PDSE2R\n")
        f.write(f"{p.isfone} {p.isfcvg} {p.dupuit}\tISFONE ISFCVG DUPUIT\n")
        f.write(f"{p.tetaf!r} {p.lump} {p.iopt}\tTETAF LUMP IOPT\n")
        f.write(f"{p.nlrelx} {p.omega!r}\tNLRELX OMEGA\n")
        f.write(f"{p.l2norm} {p.toluns!r} {p.tolswi!r} {p.ernlmx!r}\tL2NORM TOLUNS TOLSWI ERNLMX\n")
        f.write(f"{p.ituns} {p.ituns1} {p.ituns2}\tITUNS ITUNS1 ITUNS2\n")
        f.write(f"{p.isolv} {p.itmxcg} {p.tolcg!r}\tISOLV ITMXCG TOLCG\n")
        f.write(f"{p.deltat!r} {p.dtmin!r} {p.dtmax!r} {p.tmax!r}\tDELTAT DTMIN DTMAX TMAX\n")
        f.write(f"{p.dtmaga!r} {p.dtmagm!r} {p.dtreds!r} {p.dtredm!r}\tDTMAGA DTMAGM DTREDS DTREDM\n")
        timprt = list(p.timprt) or [p.tmax]
        nodvp = list(p.nodvp) or [1]
        f.write(f"{p.iprt} 2 {len(timprt)} " + " ".join(repr(float(t)) for t in timprt)
                + "\tIPRT VTKF NPRT (TIMPRT(I),I=1,NPRT)\n")
        f.write(f"{len(nodvp)} " + " ".join(str(int(i)) for i in nodvp)
                + "\tNUMVP (NODVP(I),I=1,NUMVP)\n")
        f.write("0\tNR\n0\tNUM_QOUT\n1\t(ID_QOUT(I),I=1,NUM_QOUT)\n")
    nzone, nstr = s.nzone, d.nstr
    with open(os.path.join(inp, "dem_parameters"), "w") as f:
        f.write(f"{d.delta_x!r}\n{d.delta_y!r}\n{d.factor!r}\n1\n{nzone}\t{nstr}\t25\n")
        f.write(f"{d.ivert}\t1\t{d.base!r}\n")
        f.write("\t".join(repr(float(z)) for z in d.zratio) + "\n")
    with open(os.path.join(inp, "soil"), "w") as f:
        f.write(f"{s.pmin!r}\tPMIN\n0 {s.scf!r}\tIPEAT SCF\n0.4 0.225\tCBETA0,CANG\n")
        fed = (np.array([[0.0, -4.0, -150.0, 1.0, 1.0, 1.0]]) if s.feddes is None
               else np.asarray(s.feddes, float).reshape(-1, 6))
        for row in fed:
            f.write(" ".join(repr(float(v)) for v in row) + "\tPCANA,PCREF,PCWLT,ZROOT,PZ,OMGC\n")
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
    # seepage faces: one block at TIME 0 and the same faces again at a time
    # no run reaches (SFVONE reads two blocks)
    with open(os.path.join(inp, "sfbc"), "w") as f:
        for t in (0.0, 1.0e30):
            f.write(f"{t!r}\tTIME\n{len(b.sfnod)}\tNSF\n")
            for face in b.sfnod:
                face = np.ravel(face)
                f.write(f"{len(face)}\tNNOD\n" + " ".join(str(int(i)) for i in face) + "\n")
    _raster(os.path.join(pre, "dem"), np.asarray(d.dem, float), d.west, d.south,
            d.delta_x, d.delta_y)
    if d.zone is not None:
        _raster(os.path.join(pre, "zone"), np.asarray(d.zone, float), d.west, d.south,
                d.delta_x, d.delta_y)
    if s.root_map is not None:
        _raster(os.path.join(inp, "root_map"), np.asarray(s.root_map, float), d.west,
                d.south, d.delta_x, d.delta_y)
