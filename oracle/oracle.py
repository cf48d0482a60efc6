"""ctypes wrapper of the CPU FP64 oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (oracle/cathy_oracle.cpp) restates the reference CATHY Fortran
FLOW3D path serially in double precision.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import this
module; it is the checker, never part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcathy_oracle.so")
_lib = None

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)


class OrcDem(C.Structure):
    _fields_ = [("nrow", C.c_int32), ("ncol", C.c_int32),
                ("delta_x", C.c_double), ("delta_y", C.c_double),
                ("west", C.c_double), ("south", C.c_double), ("factor", C.c_double),
                ("dem", f64p), ("zone", i32p), ("nstr", C.c_int32),
                ("zratio", f64p), ("base", C.c_double), ("ivert", C.c_int32)]


class OrcSoil(C.Structure):
    _fields_ = [("nzone", C.c_int32)] + [
        (k, f64p) for k in ("permx", "permy", "permz", "elstor", "poros", "vgn",
                            "vgrmc", "vgpsat")] + [
        ("pmin", C.c_double), ("scf", C.c_double), ("kslope", C.c_int32),
        ("tolksl", C.c_double), ("nveg", C.c_int32), ("feddes", f64p),
        ("root_map", f64p)]


class OrcParm(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("iopt", "lump", "isolv", "itmxcg", "ituns",
                                          "ituns1", "ituns2", "l2norm", "nlrelx",
                                          "isimgr")] + [
        (k, C.c_double) for k in ("tetaf", "toluns", "tolswi", "ernlmx", "tolcg",
                                   "omega", "deltat", "dtmin", "dtmax", "tmax",
                                   "dtmaga", "dtmagm", "dtreds", "dtredm",
                                   "pondh_min")] + [("precond", C.c_int32),
                                                    ("isfcvg", C.c_int32)]


class OrcBC(C.Structure):
    _fields_ = [("hspatm", C.c_int32), ("ieto", C.c_int32), ("natm", C.c_int32),
                ("atmtim", f64p), ("atminp", f64p),
                ("np", C.c_int32), ("contp", i32p), ("presc", f64p),
                ("nq", C.c_int32), ("contq", i32p), ("q", f64p),
                ("indp", C.c_int32), ("wtposition", C.c_double), ("pinit", f64p),
                ("nsf", C.c_int32), ("sfnum", i32p), ("sfnod", i32p)]


class IterRec(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("nstep", "iter", "niter", "ikmax")] + [
        (k, C.c_double) for k in ("deltat", "time", "pl2", "pinf", "pnew_ik",
                                   "pold_ik", "fl2", "finf", "lin_err", "lin_res")]


class StepRec(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("nstep", "iter", "nitert", "nback")] + [
        (k, C.c_double) for k in ("deltat", "time", "store1", "store2", "dstore",
                                   "cdstor", "vin", "cvin", "vout", "cvout",
                                   "erras", "errel", "cerras", "caeras", "sfflw",
                                   "vnd", "vnn")]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (portable flags, any host)."""
    src = os.path.join(_HERE, "cathy_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(src)):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcDem), C.POINTER(OrcSoil),
                                 C.POINTER(OrcParm), C.POINTER(OrcBC)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_sizes.argtypes = [C.c_void_p, i32p]
        L.orc_get_mesh.argtypes = [C.c_void_p, f64p, f64p, f64p, i32p, i32p, i32p, f64p, f64p]
        L.orc_get_tetra_gen3d.argtypes = [C.c_void_p, i32p]
        L.orc_step.argtypes = [C.c_void_p]
        L.orc_run.argtypes = [C.c_void_p, C.c_int32]
        L.orc_first_iteration.argtypes = [C.c_void_p, C.POINTER(IterRec)]
        L.orc_num_iter_recs.argtypes = [C.c_void_p]
        L.orc_get_iter_recs.argtypes = [C.c_void_p, C.POINTER(IterRec)]
        L.orc_num_step_recs.argtypes = [C.c_void_p]
        L.orc_get_step_recs.argtypes = [C.c_void_p, C.POINTER(StepRec)]
        L.orc_get_state.argtypes = [C.c_void_p, f64p, f64p]
        L.orc_get_qtranie.argtypes = [C.c_void_p, f64p, i32p]
        L.orc_get_seepage.argtypes = [C.c_void_p, i32p, f64p]
        L.orc_set_state.argtypes = [C.c_void_p, f64p, C.c_double, C.c_double]
        L.orc_picard_system.argtypes = [C.c_void_p, f64p, f64p, f64p, i32p]
        L.orc_vg_nodal.argtypes = [C.c_void_p, f64p, f64p, f64p, f64p, f64p]
        L.orc_asspic.argtypes = [C.c_int32, C.c_int32, i32p, i32p] + [f64p] * 15 + [C.c_int32]
        L.orc_asspic_inputs.argtypes = [C.c_void_p, i32p] + [f64p] * 12
        L.orc_symslv.restype = C.c_int32
        L.orc_symslv.argtypes = [C.c_int32, C.c_int32, C.c_int32, i32p, i32p, i32p,
                                 f64p, f64p, f64p, C.c_int32, C.c_double, C.c_int32, f64p]
        L.orc_nsyslv.restype = C.c_int32
        L.orc_nsyslv.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, i32p, i32p,
                                 i32p, f64p, f64p, f64p, C.c_int32, C.c_double, f64p]
        _lib = L
    return _lib


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(f64p)


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(i32p)


class Oracle:
    """One CATHY subsurface simulation on the CPU oracle."""

    def __init__(self, case):
        self.case = case
        self._keep = []
        d, s, p, b = case.dem, case.soil, case.parm, case.bc

        def F(a):
            arr, ptr = _f64(a)
            self._keep.append(arr)
            return ptr

        def I(a):
            arr, ptr = _i32(a)
            self._keep.append(arr)
            return ptr

        dem = OrcDem(nrow=d.nrow, ncol=d.ncol, delta_x=d.delta_x, delta_y=d.delta_y,
                     west=d.west, south=d.south, factor=d.factor,
                     dem=F(d.dem.reshape(-1)),
                     zone=I(d.zone.reshape(-1)) if d.zone is not None else None,
                     nstr=d.nstr, zratio=F(d.zratio), base=d.base, ivert=d.ivert)
        soil = OrcSoil(nzone=s.nzone, pmin=s.pmin, scf=s.scf, kslope=s.kslope,
                       tolksl=s.tolksl)
        for k in ("permx", "permy", "permz", "elstor", "poros", "vgn", "vgrmc", "vgpsat"):
            setattr(soil, k, F(getattr(s, k).reshape(-1)))
        fed = getattr(s, "feddes", None)
        if fed is not None:
            fed = np.asarray(fed, dtype=np.float64).reshape(-1, 6)
            soil.nveg = fed.shape[0]
            soil.feddes = F(fed.reshape(-1))
        rmap = getattr(s, "root_map", None)
        if rmap is not None:
            soil.root_map = F(np.asarray(rmap, dtype=np.float64).reshape(-1))
        parm = OrcParm(**{k: getattr(p, k) for k, _ in OrcParm._fields_})
        pinit = b.pinit if b.pinit is not None else np.zeros(1)
        bc = OrcBC(hspatm=b.hspatm, ieto=b.ieto, natm=len(b.atmtim),
                   atmtim=F(b.atmtim), atminp=F(np.asarray(b.atminp).reshape(-1)),
                   np=len(b.contp), contp=I(b.contp if len(b.contp) else np.zeros(1)),
                   presc=F(b.presc if len(b.presc) else np.zeros(1)),
                   nq=len(b.contq), contq=I(b.contq if len(b.contq) else np.zeros(1)),
                   q=F(b.q if len(b.q) else np.zeros(1)),
                   indp=b.indp, wtposition=b.wtposition, pinit=F(pinit))
        faces = [np.asarray(f, dtype=np.int32).reshape(-1) for f in getattr(b, "sfnod", [])]
        if faces:
            bc.nsf = len(faces)
            bc.sfnum = I(np.array([len(f) for f in faces], np.int32))
            bc.sfnod = I(np.concatenate(faces))
        self.nsfn = int(sum(len(f) for f in faces))
        self.h = lib().orc_create(C.byref(dem), C.byref(soil), C.byref(parm), C.byref(bc))
        if not self.h:
            raise RuntimeError("oracle: mesh construction failed")
        sz = (C.c_int32 * 5)()
        lib().orc_sizes(self.h, sz)
        self.n, self.nt, self.nnod, self.ntri, self.nterm = list(sz)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def mesh(self):
        n, nt = self.n, self.nt
        x, y, z = np.zeros(n), np.zeros(n), np.zeros(n)
        tetra = np.zeros(5 * nt, np.int32)
        topol = np.zeros(n + 1, np.int32)
        ja = np.zeros(self.nterm, np.int32)
        arenod, volnod = np.zeros(self.nnod), np.zeros(n)
        lib().orc_get_mesh(self.h, *[_f64(a)[1] for a in (x, y, z)], _i32(tetra)[1],
                           _i32(topol)[1], _i32(ja)[1], _f64(arenod)[1], _f64(volnod)[1])
        return dict(x=x, y=y, z=z, tetra=tetra.reshape(nt, 5), topol=topol, ja=ja,
                    arenod=arenod, volnod=volnod)

    def tetra_gen3d(self):
        t = np.zeros(5 * self.nt, np.int32)
        lib().orc_get_tetra_gen3d(self.h, _i32(t)[1])
        return t.reshape(self.nt, 5)

    def first_iteration(self):
        r = IterRec()
        lib().orc_first_iteration(self.h, C.byref(r))
        return {k: getattr(r, k) for k, _ in IterRec._fields_}

    def step(self):
        return lib().orc_step(self.h)

    def run(self, max_steps=10 ** 9):
        return lib().orc_run(self.h, max_steps)

    def iter_records(self):
        k = lib().orc_num_iter_recs(self.h)
        arr = (IterRec * max(k, 1))()
        lib().orc_get_iter_recs(self.h, arr)
        return [{f: getattr(arr[i], f) for f, _ in IterRec._fields_} for i in range(k)]

    def step_records(self):
        k = lib().orc_num_step_recs(self.h)
        arr = (StepRec * max(k, 1))()
        lib().orc_get_step_recs(self.h, arr)
        return [{f: getattr(arr[i], f) for f, _ in StepRec._fields_} for i in range(k)]

    def state(self):
        p = np.zeros(self.n)
        td = np.zeros(2)
        lib().orc_get_state(self.h, _f64(p)[1], _f64(td)[1])
        return p, float(td[0]), float(td[1])

    def seepage(self):
        """SFEX and SFQ, one entry per seepage-face node in input order."""
        ex = np.zeros(max(self.nsfn, 1), dtype=np.int32)
        q = np.zeros(max(self.nsfn, 1))
        lib().orc_get_seepage(self.h, ex.ctypes.data_as(i32p), _f64(q)[1])
        return ex[: self.nsfn], q[: self.nsfn]

    def qtranie(self):
        """QTRANIE of the current time step (n) and VEG_TYPE (nnod)."""
        q = np.zeros(self.n)
        vt = np.zeros(self.nnod, dtype=np.int32)
        lib().orc_get_qtranie(self.h, _f64(q)[1], vt.ctypes.data_as(i32p))
        return q, vt

    def set_state(self, ptimep, time, deltat):
        a, ptr = _f64(ptimep)
        lib().orc_set_state(self.h, ptr, time, deltat)

    def picard_system(self):
        c1 = np.zeros(self.nterm)
        tn, xt5 = np.zeros(self.n), np.zeros(self.n)
        dm = np.zeros(self.n, np.int32)
        lib().orc_picard_system(self.h, _f64(c1)[1], _f64(tn)[1], _f64(xt5)[1], _i32(dm)[1])
        return c1, tn, xt5, dm

    def asspic_inputs(self):
        """ASSPIC's arguments at the current state (call after picard_system):
        the reference's arrays in memory order."""
        nt = self.nt
        tetja = np.zeros(16 * nt, np.int32)
        lmass = np.zeros(16)
        e = [np.zeros(nt) for _ in range(5)]
        nzs = len(self.case.soil.permx.reshape(-1))
        p = [np.zeros(nzs) for _ in range(3)]
        g = [np.zeros(4 * nt) for _ in range(3)]
        et1e, pel, ckrwe, volu, volur = e
        lib().orc_asspic_inputs(self.h, _i32(tetja)[1], _f64(lmass)[1], _f64(et1e)[1],
                                _f64(pel)[1], *[_f64(a)[1] for a in p], _f64(ckrwe)[1],
                                _f64(volu)[1], _f64(volur)[1], *[_f64(a)[1] for a in g])
        return dict(tetra=self.mesh()["tetra"], tetja=tetja, lmass=lmass, et1e=et1e, pel=pel,
                    permx=p[0], permy=p[1], permz=p[2], ckrwe=ckrwe, volu=volu, volur=volur,
                    bi=g[0], ci=g[1], di=g[2], ntri=self.ntri,
                    maxstr=self.case.dem.nstr)

    def vg_nodal(self, psi):
        psi, pp = _f64(psi)
        out = [np.zeros(self.n) for _ in range(4)]
        lib().orc_vg_nodal(self.h, pp, *[_f64(o)[1] for o in out])
        return dict(sw=out[0], ckrw=out[1], etai=out[2], et2=out[3])


def symslv(topol, ja, coef1, b, noddir, itmxcg=500, tolcg=1e-10, jacobi=False):
    """Reference SYMSLV (IC(0)- or Jacobi-PCG) on 1-based symmetric upper CSR."""
    n = len(topol) - 1
    x = np.zeros(n)
    er = np.zeros(2)
    nd = np.asarray(noddir, np.int32)
    niter = lib().orc_symslv(n, len(ja), len(nd), _i32(nd if len(nd) else np.zeros(1))[1],
                             _i32(ja)[1], _i32(topol)[1], _f64(x)[1], _f64(b)[1],
                             _f64(coef1)[1], itmxcg, tolcg, int(jacobi), _f64(er)[1])
    return x, int(niter), float(er[0]), float(er[1])


def nsyslv(topol, ja, coef1, b, noddir, isolv=0, itmxcg=500, tolcg=1e-10):
    """Reference NSYSLV (ISOLV 0 ILU(0)-BiCGSTAB, -5 Jacobi-BiCGSTAB), full CSR."""
    n = len(topol) - 1
    x = np.zeros(n)
    er = np.zeros(2)
    nd = np.asarray(noddir, np.int32)
    niter = lib().orc_nsyslv(isolv, n, len(ja), len(nd),
                             _i32(nd if len(nd) else np.zeros(1))[1], _i32(ja)[1],
                             _i32(topol)[1], _f64(x)[1], _f64(b)[1], _f64(coef1)[1],
                             itmxcg, tolcg, _f64(er)[1])
    return x, int(niter), float(er[0]), float(er[1])


def asspic(tetra, tetja, lmass, coef1, coef2, coef4, et1e, pel, permx, permy, permz,
           ckrwe, volu, volur, bi, ci, di, ntri, maxstr):
    """Reference ASSPIC on the caller's arrays (same layout as the drop-in);
    returns accumulated copies of COEF1, COEF2, COEF4."""
    tetra = np.ascontiguousarray(tetra, np.int32).reshape(-1)
    tetja = np.ascontiguousarray(tetja, np.int32).reshape(-1)
    c1, c2, c4 = (np.array(a, np.float64) for a in (coef1, coef2, coef4))
    arrs = [np.ascontiguousarray(a, np.float64).reshape(-1)
            for a in (lmass, et1e, pel, permx, permy, permz, ckrwe, volu, volur, bi, ci, di)]
    lm, a1, a2, px, py, pz, kr, vo, vr, b, c, d = arrs
    lib().orc_asspic(len(tetra) // 5, ntri, _i32(tetra)[1], _i32(tetja)[1], _f64(lm)[1],
                     _f64(c1)[1], _f64(c2)[1], _f64(c4)[1], _f64(a1)[1], _f64(a2)[1],
                     _f64(px)[1], _f64(py)[1], _f64(pz)[1], _f64(kr)[1], _f64(vo)[1],
                     _f64(vr)[1], _f64(b)[1], _f64(c)[1], _f64(d)[1], maxstr)
    return c1, c2, c4
