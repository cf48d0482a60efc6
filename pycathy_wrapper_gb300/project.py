"""Reader for a CATHY project directory (the files pyCATHY writes).

Restates the input semantics of the reference's ``datin.f`` for the
subsurface solver (parm :81-117, DEM/zone rasters via RAST_INPUT_DEM /
RAST_INPUT_LZ :189-257, dem_parameters :195-266, ic :380-405, soil
:421-517) plus the atmospheric (``atmone.f``) and non-atmospheric BC files
(``bcone.f``; constant in time: later blocks must repeat the first).  The result is a
:class:`~pycathy_wrapper_gb300.inputs.Case`, so a pyCATHY project can be run
on the GPU without changing how the project is written.
"""
from __future__ import annotations

import os
import re

import numpy as np

from .inputs import BC, Case, Dem, Parm, Soil

_num = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eEdD][+-]?\d+)?$")


def _nums(line):
    out = []
    for tok in line.replace(",", " ").split():
        if _num.match(tok):
            out.append(float(tok.replace("d", "e").replace("D", "e")))
        else:
            break
    return out


def _lines(path):
    with open(path) as f:
        return [ln for ln in f.read().splitlines()]


def read_raster(path):
    """GRASS-ASCII raster with a 6-line header (north/south/east/west/rows/cols)."""
    ls = _lines(path)
    hdr = {}
    for ln in ls[:6]:
        k, v = ln.split(":")
        hdr[k.strip()] = float(v)
    nrow, ncol = int(hdr["rows"]), int(hdr["cols"])
    vals = np.array(" ".join(ls[6:]).replace("D", "E").split(), dtype=float)
    return vals[: nrow * ncol].reshape(nrow, ncol), hdr


def read_parm(path) -> Parm:
    ls = [ln for ln in _lines(path) if ln.strip()]
    v = [_nums(ln) for ln in ls]
    p = Parm()
    p.isimgr = int(v[1][0])
    p.pondh_min = v[1][1]
    p.kslope = int(v[2][0])
    p.tetaf, p.lump, p.iopt = v[6][0], int(v[6][1]), int(v[6][2])
    p.nlrelx, p.omega = int(v[7][0]), v[7][1]
    if p.iopt == 2 and p.isolv not in (0, -5):
        raise ValueError("IOPT = 2 with ISOLV other than 0 or -5 is not supported")
    if p.nlrelx not in (0, 1):
        raise ValueError("NLRELX = 2 (variable relaxation, relxom.f) is not supported")
    p.l2norm, p.toluns, p.tolswi, p.ernlmx = int(v[8][0]), v[8][1], v[8][2], v[8][3]
    p.ituns, p.ituns1, p.ituns2 = int(v[9][0]), int(v[9][1]), int(v[9][2])
    p.isolv, p.itmxcg, p.tolcg = int(v[10][0]), int(v[10][1]), v[10][2]
    p.deltat, p.dtmin, p.dtmax, p.tmax = v[11][:4]
    p.dtmaga, p.dtmagm, p.dtreds, p.dtredm = v[12][:4]
    p.tolksl = v[2][1]
    p.isfone, p.isfcvg, p.dupuit = (int(x) for x in v[5][:3])
    p.iprt1 = int(v[0][0])
    # IPRT VTKF NPRT (TIMPRT(I),I=1,NPRT) then NUMVP (NODVP(I),I=1,NUMVP):
    # list-directed reads (datin.f:118-119), so a list may run on over
    # several lines
    k = 13
    if len(v) > k and len(v[k]) >= 3:
        p.iprt, nprt = int(v[k][0]), int(v[k][2])
        vals = list(v[k][3:])
        while len(vals) < nprt and k + 1 < len(v):
            k += 1
            vals += v[k]
        p.timprt = [float(t) for t in vals[:nprt]]
        k += 1
        if k < len(v) and v[k]:
            numvp = int(v[k][0])
            ids = list(v[k][1:])
            while len(ids) < numvp and k + 1 < len(v):
                k += 1
                ids += v[k]
            p.nodvp = [int(i) for i in ids[:numvp]]
    return p


def read_project(prj: str) -> Case:
    """Read ``prj/input/*`` and ``prj/prepro/*`` into a Case."""
    inp = lambda f: os.path.join(prj, "input", f)
    pre = lambda f: os.path.join(prj, "prepro", f)
    parm = read_parm(inp("parm"))
    # dem_parameters: delta_x, delta_y, factor, dostep, nzone nstr n1,
    # ivert isp base, zratio
    dp = [_nums(ln) for ln in _lines(inp("dem_parameters")) if _nums(ln)]
    delta_x, delta_y, factor = dp[0][0], dp[1][0], dp[2][0]
    nzone, nstr = int(dp[4][0]), int(dp[4][1])
    ivert, base = int(dp[5][0]), dp[5][2]
    if ivert not in (0, 1, 2, 4):
        # IVERT 3 reads a per-node depth map (gen3d.f:67-68)
        raise ValueError(f"IVERT = {ivert} is not supported (0, 1, 2 and 4 are)")
    zr = np.array(dp[6][:nstr])
    dem_map, hdr = read_raster(pre("dem"))
    zone_map = None
    if os.path.exists(pre("zone")):
        z, _ = read_raster(pre("zone"))
        zone_map = np.rint(z).astype(np.int32)
    dem = Dem(dem=dem_map, delta_x=delta_x, delta_y=delta_y, zratio=zr,
              base=base, ivert=ivert, zone=zone_map, factor=factor,
              west=hdr.get("west", 0.0), south=hdr.get("south", 0.0))
    # vegetation types (datin.f:221-233): the root map's largest type is
    # the number of Feddes lines in the soil file (datin.f:424-428)
    nveg = 1
    root_map = None
    if os.path.exists(inp("root_map")):
        root_map, _ = read_raster(inp("root_map"))
        nveg = max(1, int(np.max(root_map)))
    sl = [ln for ln in _lines(inp("soil")) if _nums(ln)]
    pmin = _nums(sl[0])[0]
    ipeat, scf = int(_nums(sl[1])[0]), _nums(sl[1])[1]
    if ipeat != 0:
        raise ValueError("IPEAT = 1 (peat soil deformation) is not supported")
    # nudging (input/nudging: NUDFLAG NUDN WFLAG) adds terms this solver
    # does not model
    if os.path.exists(inp("nudging")):
        nud = [_nums(ln) for ln in _lines(inp("nudging")) if _nums(ln)]
        if nud and len(nud[0]) > 1 and int(nud[0][1]) > 0:
            raise ValueError("nudging observations (NUDN > 0) are not supported")
    feddes = np.array([_nums(sl[3 + v])[:6] for v in range(nveg)], dtype=float)
    ivghu = int(_nums(sl[3 + nveg])[0])
    if ivghu != 0:
        raise ValueError("only IVGHU=0 (van Genuchten) soils are supported")
    rows = np.array([_nums(ln)[:8] for ln in sl[8 + nveg: 8 + nveg + nstr * nzone]])
    rows = rows.reshape(nstr, nzone, 8).transpose(1, 0, 2)  # (zone, layer, 8)
    soil = Soil(permx=rows[..., 0].copy(), permy=rows[..., 1].copy(),
                permz=rows[..., 2].copy(), elstor=rows[..., 3].copy(),
                poros=rows[..., 4].copy(), vgn=rows[..., 5].copy(),
                vgrmc=rows[..., 6].copy(), vgpsat=rows[..., 7].copy(),
                pmin=pmin, scf=scf, kslope=parm.kslope, tolksl=parm.tolksl,
                feddes=feddes, root_map=root_map)
    # initial conditions
    il = [ln for ln in _lines(inp("ic")) if ln.strip()]
    head = _nums(il[0])
    indp = int(head[0])
    ipond = int(head[1]) if len(head) > 1 else 0
    if ipond != 0 and parm.isimgr == 2:
        # datin.f:380-410: ponded initial heads, read only with surface
        # routing (ISIMGR = 2), which this solver does not model
        raise ValueError("IPOND != 0 (ponded initial conditions) needs surface routing")
    bc = BC(indp=indp)
    if indp in (3, 4):
        bc.wtposition = _nums(il[1])[0]
    elif indp == 0:
        bc.pinit = np.array([_nums(il[1])[0]])
    elif indp == 1:
        bc.pinit = np.array(" ".join(il[1:]).split(), dtype=float)
    # atmospheric forcing
    al = [ln for ln in _lines(inp("atmbc")) if ln.strip()]
    h = _nums(al[0])
    bc.hspatm, bc.ieto = int(h[0]), int(h[1])
    toks = []
    for ln in al[1:]:
        toks.extend(_nums(ln))
    times, vals = [], []
    i = 0
    per = 1 if bc.hspatm != 0 else None
    while i < len(toks):
        times.append(toks[i])
        i += 1
        if per is None:
            # spatially variable: the rest of the block until the next time is
            # NNOD values; NNOD is the number of active DEM cell corners
            nnod = _count_nodes(dem_map)
            per = nnod
        vals.append(toks[i:i + per])
        i += per
    bc.atmtim = np.array(times)
    bc.atminp = np.array(vals) if per != 1 else np.array([v[0] for v in vals])
    parm_dir = _read_bc_list(inp("nansfdirbc"), parm.tmax)
    if parm_dir is not None:
        bc.contp, bc.presc = parm_dir
    neu = _read_bc_list(inp("nansfneubc"), parm.tmax)
    if neu is not None:
        bc.contq, bc.q = neu
    if os.path.exists(inp("sfbc")):
        bc.sfnod = read_sfbc(inp("sfbc"), parm.tmax)
    if bc.sfnod and (parm.isfone != 0 or parm.dupuit != 0):
        # conver.f:88-99 and sfinit.f:35-41 stop on these
        raise ValueError("seepage faces need ISFONE = 0 and DUPUIT = 0")
    return Case(dem, soil, parm, bc, name=os.path.basename(os.path.normpath(prj)))


def read_sfbc(path, tmax=np.inf):
    """``input/sfbc`` as SFVONE/SFVNXT read it (sfvone.f, sfvnxt.f): blocks
    of TIME, NSF and per face a line with its node count followed by the
    node list (list-directed: it may run over several lines, the rest of its
    last line is skipped).  A block takes effect once TIME exceeds its time;
    blocks at or after TMAX never do.  Only a time-invariant set of faces is
    supported: every effective block must repeat the first one."""
    rows = [_nums(ln) for ln in _lines(path)]
    rows = [r for r in rows if r]
    k = 0

    def first():
        nonlocal k
        v = rows[k][0]
        k += 1
        return v

    blocks = []
    while k < len(rows):
        t = first()
        if k >= len(rows):
            break
        nsf = int(first())
        faces = []
        for _ in range(nsf):
            cnt = int(first())
            ids = []
            while len(ids) < cnt:
                ids += rows[k]
                k += 1
            faces.append(np.array(ids[:cnt], dtype=np.int32))
        blocks.append((t, faces))
    if not blocks or not any(faces for _, faces in blocks):
        return []  # no seepage face at any time
    if blocks[0][0] > 0.0:
        raise ValueError("input/sfbc: the first block must start at TIME = 0")
    ref = blocks[0][1]
    for t, faces in blocks[1:]:
        if t >= tmax:
            continue
        same = len(faces) == len(ref) and all(np.array_equal(a, b) for a, b in zip(faces, ref))
        if not same:
            raise ValueError("input/sfbc: time-varying seepage faces are not supported")
    return ref


def _count_nodes(dem_map):
    nrow, ncol = dem_map.shape
    act = np.zeros((nrow + 1, ncol + 1), bool)
    on = dem_map != 0
    act[:-1, :-1] |= on
    act[1:, :-1] |= on
    act[1:, 1:] |= on
    act[:-1, 1:] |= on
    return int(act.sum())


def _read_bc_list(path, tmax=np.inf):
    """A nansfdirbc / nansfneubc file as BCONE/BCNXT read it (bcone.f):
    blocks of ``time`` / ``NDIR NDIRC`` (or ``ZERO NQ``) / node ids /
    values.  The solver holds these conditions constant, so every block
    that takes effect before TMAX must repeat the first one (BCNXT would
    interpolate between differing blocks)."""
    if not os.path.exists(path):
        return None
    toks = []
    for ln in _lines(path):
        toks.extend(_nums(ln))
    blocks, i = [], 0
    while i + 2 < len(toks):
        t, n1, n2 = toks[i], int(toks[i + 1]), int(toks[i + 2])
        cnt = n1 + n2
        ids = np.array(toks[i + 3:i + 3 + cnt], dtype=np.int32)
        vals = np.array(toks[i + 3 + cnt:i + 3 + 2 * cnt], dtype=float)
        if len(vals) < cnt:
            vals = np.zeros(cnt)
        blocks.append((t, ids, vals))
        i += 3 + 2 * cnt
    if not blocks or len(blocks[0][1]) == 0:
        if any(len(b[1]) for b in blocks if b[0] < tmax):
            raise ValueError(f"{path}: time-varying boundary conditions are not supported")
        return None
    _, ids0, vals0 = blocks[0]
    for t, ids, vals in blocks[1:]:
        if t < tmax and not (np.array_equal(ids, ids0) and np.array_equal(vals, vals0)):
            raise ValueError(f"{path}: time-varying boundary conditions are not supported")
    return ids0, vals0