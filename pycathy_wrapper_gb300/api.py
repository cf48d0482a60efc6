"""Python API over the C ABI.

* :class:`Simulation` owns the device state of one CATHY simulation or of a
  whole ensemble (one member per :class:`~pycathy_wrapper_gb300.inputs.Case`)
  and advances it on the GPU.  It is the batched replacement of running one
  ``./cathy`` process per member (pyCATHY ``CATHY.run_processor``,
  cathy_tools.py:593, and ``DA._run_ensemble_hydrological_model``,
  DA/cathy_DA.py:1373).
* :func:`symslv`, :func:`nsyslv`, :func:`asspic` expose the Fortran
  subroutine drop-ins with the reference's argument meaning (1-based CSR
  contents).
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence, Union

import numpy as np

from . import _lib
from ._lib import check, f64p, i32p
from .inputs import Case

PRECISION_FP64 = 0
PRECISION_MIXED = 1


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class _Keep:
    def __init__(self):
        self.refs = []

    def f(self, a):
        a = _f64(a)
        self.refs.append(a)
        return _ptr(a, f64p)

    def i(self, a):
        a = _i32(a)
        self.refs.append(a)
        return _ptr(a, i32p)


def _member(case: Case, keep: _Keep) -> _lib.Member:
    d, s, p, b = case.dem, case.soil, case.parm, case.bc
    mem = _lib.Member()
    mem.dem = _lib.Dem(nrow=d.nrow, ncol=d.ncol, delta_x=d.delta_x, delta_y=d.delta_y,
                       west=d.west, south=d.south, factor=d.factor,
                       dem=keep.f(d.dem.reshape(-1)),
                       zone=keep.i(d.zone.reshape(-1)) if d.zone is not None else None,
                       nstr=d.nstr, zratio=keep.f(d.zratio), base=d.base, ivert=d.ivert)
    soil = _lib.Soil(nzone=s.nzone, pmin=s.pmin, scf=s.scf, kslope=s.kslope, tolksl=s.tolksl)
    for k in ("permx", "permy", "permz", "elstor", "poros", "vgn", "vgrmc", "vgpsat"):
        setattr(soil, k, keep.f(getattr(s, k).reshape(-1)))
    if s.feddes is not None:
        fed = np.asarray(s.feddes, dtype=np.float64).reshape(-1, 6)
        soil.nveg = fed.shape[0]
        soil.feddes = keep.f(fed.reshape(-1))
    if s.root_map is not None:
        soil.root_map = keep.f(np.asarray(s.root_map, dtype=np.float64).reshape(-1))
    mem.soil = soil
    mem.parm = _lib.Parm(**{k: getattr(p, k) for k, _ in _lib.Parm._fields_})
    pinit = b.pinit if b.pinit is not None else np.zeros(1)
    z1 = np.zeros(1)
    mem.bc = _lib.BC(hspatm=b.hspatm, ieto=b.ieto, natm=len(b.atmtim),
                     atmtim=keep.f(b.atmtim), atminp=keep.f(np.asarray(b.atminp).reshape(-1)),
                     np=len(b.contp), contp=keep.i(b.contp if len(b.contp) else z1),
                     presc=keep.f(b.presc if len(b.presc) else z1),
                     nq=len(b.contq), contq=keep.i(b.contq if len(b.contq) else z1),
                     q=keep.f(b.q if len(b.q) else z1),
                     indp=b.indp, wtposition=b.wtposition, pinit=keep.f(pinit))
    faces = [np.asarray(f, dtype=np.int32).reshape(-1) for f in b.sfnod]
    if faces:
        mem.bc.nsf = len(faces)
        mem.bc.sfnum = keep.i(np.array([len(f) for f in faces], np.int32))
        mem.bc.sfnod = keep.i(np.concatenate(faces))
    return mem


class Simulation:
    """CATHY subsurface simulation(s) on one GPU.

    ``cases`` is one Case or a list (an ensemble: members may differ in mesh
    and soil but share IOPT, LUMP and the preconditioner).  ``precision`` 0
    runs FP64 everywhere (the reference's arithmetic); 1 assembles and runs
    the Krylov iterations in FP32 inside an FP64 residual/refinement loop.
    ``inner_tol`` is the FP32 Krylov solve's relative tolerance (the larger
    of it and TOLCG is used): at 1e-8 the FP32 path takes the oracle's time
    steps on every tested member; at 1e-6 some members drift to different
    (equally converged) iterates and, over a day, a different step sequence.
    """

    def __init__(self, cases: Union[Case, Sequence[Case]], precision: int = 0,
                 device: int = 0, inner_maxit: int = 200, inner_tol: float = 1e-8,
                 graphs: bool = True):
        self.L = _lib.load()
        self.cases: List[Case] = [cases] if isinstance(cases, Case) else list(cases)
        keep = _Keep()
        arr = (_lib.Member * len(self.cases))()
        for m, c in enumerate(self.cases):
            arr[m] = _member(c, keep)
        opts = _lib.Opts(precision=precision, device=device, inner_maxit=inner_maxit,
                         inner_tol=inner_tol, verbose=0, graphs=1 if graphs else 0)
        h = C.c_void_p()
        check(self.L.cathy_gb300_create(len(self.cases), arr, C.byref(opts), C.byref(h)),
              "cathy_gb300_create")
        self.h = h
        self._keep = keep
        self.sizes = []
        for m in range(len(self.cases)):
            out = (C.c_int32 * 5)()
            check(self.L.cathy_gb300_sizes(self.h, m, out), "sizes")
            self.sizes.append(dict(n=out[0], nt=out[1], nnod=out[2], ntri=out[3], nnz=out[4]))

    def close(self):
        if getattr(self, "h", None):
            self.L.cathy_gb300_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def nmembers(self):
        return len(self.cases)

    def step(self) -> int:
        """Advance every running member by one accepted time step."""
        na = C.c_int32()
        check(self.L.cathy_gb300_step(self.h, C.byref(na)), "cathy_gb300_step")
        return na.value

    def run(self, max_steps: int = 0) -> int:
        ns = C.c_int32()
        check(self.L.cathy_gb300_run(self.h, max_steps, C.byref(ns)), "cathy_gb300_run")
        return ns.value

    def state(self, m: int = 0):
        n = self.sizes[m]["n"]
        p = np.zeros(n)
        t, dt, stt = C.c_double(), C.c_double(), C.c_int32()
        check(self.L.cathy_gb300_get_state(self.h, m, _ptr(p, f64p), C.byref(t), C.byref(dt),
                                           C.byref(stt)), "get_state")
        return p, t.value, dt.value, stt.value

    def saturation(self, m: int = 0):
        """Water saturation of member m at its current heads (the SW array of
        the reference's ``sw`` output, detout.f:44-45)."""
        sw = np.zeros(self.sizes[m]["n"])
        check(self.L.cathy_gb300_get_saturation(self.h, m, _ptr(sw, f64p)), "get_saturation")
        return sw

    def seepage(self, m: int = 0):
        """SFEX (exit-point flags) and SFQ (back-calculated fluxes) of member
        m's seepage-face nodes, in the order of its ``bc.sfnod`` faces."""
        k = int(sum(len(f) for f in self.cases[m].bc.sfnod))
        ex = np.zeros(max(k, 1), np.int32)
        q = np.zeros(max(k, 1))
        check(self.L.cathy_gb300_get_seepage(self.h, m, _ptr(ex, i32p), _ptr(q, f64p)),
              "get_seepage")
        return ex[:k], q[:k]

    def set_state(self, m: int, ptimep, time: float, deltat: float):
        p = _f64(ptimep)
        check(self.L.cathy_gb300_set_state(self.h, m, _ptr(p, f64p), time, deltat), "set_state")

    def num_records(self, m: int = 0):
        """(iteration records, accepted steps) of member m so far."""
        ni, ns = C.c_int32(), C.c_int32()
        check(self.L.cathy_gb300_num_records(self.h, m, C.byref(ni), C.byref(ns)), "records")
        return ni.value, ns.value

    def records(self, m: int = 0):
        ni, ns = C.c_int32(), C.c_int32()
        check(self.L.cathy_gb300_num_records(self.h, m, C.byref(ni), C.byref(ns)), "records")
        ir = (_lib.IterRec * max(ni.value, 1))()
        sr = (_lib.StepRec * max(ns.value, 1))()
        check(self.L.cathy_gb300_get_records(self.h, m, ir, sr), "records")
        its = [{k: getattr(ir[i], k) for k, _ in _lib.IterRec._fields_} for i in range(ni.value)]
        sts = [{k: getattr(sr[i], k) for k, _ in _lib.StepRec._fields_} for i in range(ns.value)]
        return its, sts

    def mesh(self, m: int = 0):
        s = self.sizes[m]
        x, y, z = np.zeros(s["n"]), np.zeros(s["n"]), np.zeros(s["n"])
        tetra = np.zeros(5 * s["nt"], np.int32)
        rowptr = np.zeros(s["n"] + 1, np.int32)
        cols = np.zeros(s["nnz"], np.int32)
        check(self.L.cathy_gb300_get_mesh(self.h, m, _ptr(x, f64p), _ptr(y, f64p), _ptr(z, f64p),
                                          _ptr(tetra, i32p), _ptr(rowptr, i32p),
                                          _ptr(cols, i32p)), "get_mesh")
        return dict(x=x, y=y, z=z, tetra=tetra.reshape(-1, 5), rowptr=rowptr, cols=cols)

    def picard_system(self, m: int = 0):
        s = self.sizes[m]
        vals, rhs, xt5 = np.zeros(s["nnz"]), np.zeros(s["n"]), np.zeros(s["n"])
        dm = np.zeros(s["n"], np.int32)
        check(self.L.cathy_gb300_picard_system(self.h, m, _ptr(vals, f64p), _ptr(rhs, f64p),
                                               _ptr(xt5, f64p), _ptr(dm, i32p)), "picard_system")
        return vals, rhs, xt5, dm

    def reset(self):
        """Restore every member to its initial condition (device-side)."""
        check(self.L.cathy_gb300_reset(self.h), "cathy_gb300_reset")

    def profile(self, enable: int = -1):
        """Live SpMV timing: enable=1 starts (and zeroes) it, 0 stops, -1 reads.
        Returns (device ms, launches, algorithmic bytes) accumulated so far."""
        ms, bts = C.c_double(), C.c_double()
        n = C.c_int64()
        check(self.L.cathy_gb300_profile(self.h, enable, C.byref(ms), C.byref(n), C.byref(bts)),
              "cathy_gb300_profile")
        return ms.value, n.value, bts.value

    def attach_learned(self, model, mode: int = 2):
        """Attach a :class:`~pycathy_wrapper_gb300.learned.LearnedPreconditioner`
        (mode 1 train on the plain solves, 2 use with plain fallback, 0 detach)."""
        h = model.handle if model is not None else None
        check(self.L.cathy_gb300_attach_learned(self.h, h, int(mode)), "attach_learned")
        self._lp = model

    def learned_stats(self):
        out = (C.c_double * 6)()
        check(self.L.cathy_gb300_learned_stats(self.h, out, 6), "learned_stats")
        return dict(learned_solves=out[0], learned_iters=out[1], plain_solves=out[2],
                    plain_iters=out[3], train_steps=out[4], last_loss=out[5])

    def timers(self):
        """Host-side phase timers of the time stepping."""
        out = (C.c_double * 72)()
        check(self.L.cathy_gb300_timers(self.h, out, 72), "cathy_gb300_timers")
        k = ("macro_iterations", "graph_launches", "graph_builds", "host_prep_ms",
             "device_wait_ms", "host_decision_ms", "gpu_ms", "graph_gpu_ms")
        d = {a: out[i] for i, a in enumerate(k)}
        d["by_log2_rows"] = {b: (out[8 + 2 * b], out[9 + 2 * b]) for b in range(32)
                             if out[8 + 2 * b] > 0}
        return d

    def autotune(self, nrep: int = 10):
        """Time the assembly (mode 0: inputs read directly, 1: staged in
        shared memory by bulk copies, 2: staged with 8 lanes per row;
        resident blocks per SM) and stream-SpMV schedules on the running
        members and keep the fastest (cached per GPU and size class;
        nrep <= 0 reuses a cached choice).
        Returns dict(asm_blocks, spmv_blocks, asm_staged (the mode),
        spmv_staged, asm_ms, spmv_ms)."""
        sc = (C.c_int32 * 4)()
        ms = (C.c_double * 2)()
        check(self.L.cathy_gb300_autotune(self.h, int(nrep), sc, ms), "autotune")
        return dict(asm_blocks=sc[0], spmv_blocks=sc[1], asm_staged=int(sc[2]),
                    spmv_staged=int(sc[3]), asm_ms=ms[0], spmv_ms=ms[1])

    def set_schedule(self, asm_blocks: int, spmv_blocks: int, asm_staged: int = 0,
                     spmv_staged: int = 0):
        check(self.L.cathy_gb300_set_schedule(self.h, int(asm_blocks), int(spmv_blocks),
                                              int(asm_staged), int(spmv_staged)),
              "set_schedule")

    PHASES = ("UNSAT CHARACTERISTICS", "INIT. OF SYSTEM MATRICES", "LOCAL SYSTEM ASSEMBLY",
              "RHS CALCULATION W/O BC'S", "GLOBAL LHS SYSTEM MATRIX", "BC CONTRIBUTIONS TO RHS",
              "LINEAR SOLVER & RESIDUAL", "DIR. RESETTING AND DIFMAX",
              "B-FLX, M-BAL, SW, & EX-PT")

    def phase_timers(self, enable: int = -1):
        """GPU ms per phase bucket of the reference's risul summary (enable 1
        starts timing, 0 stops it, -1 reads); a dict name -> ms."""
        out = (C.c_double * 9)()
        check(self.L.cathy_gb300_phase_timers(self.h, int(enable), out, 9), "phase_timers")
        return {k: out[i] for i, k in enumerate(self.PHASES)}

    def time_assembly(self, nrep: int = 10):
        """Mean device time (ms) of the FP32 assembly over the members that
        iterated last, its algorithmic bytes and rows (see the C header)."""
        ms, b = C.c_double(), C.c_double()
        r = C.c_int64()
        check(self.L.cathy_gb300_time_assembly(self.h, int(nrep), C.byref(ms), C.byref(b),
                                               C.byref(r)), "time_assembly")
        return ms.value, b.value, r.value

    def stats(self):
        ms = C.c_double()
        la, li, nl = C.c_int64(), C.c_int64(), C.c_int64()
        check(self.L.cathy_gb300_stats(self.h, C.byref(ms), C.byref(la), C.byref(li),
                                       C.byref(nl)), "stats")
        return dict(gpu_ms=ms.value, launches=la.value, lin_iters=li.value, nl_iters=nl.value)


def build_mesh(case: Case, iopt: int = 1):
    """Host-side mesh of a case as the GPU engine builds it (no device)."""
    L = _lib.load()
    keep = _Keep()
    mem = _member(case, keep)
    out = (C.c_int32 * 5)()
    check(L.cathy_gb300_mesh(C.byref(mem.dem), iopt, out, None, None, None, None, None, None),
          "cathy_gb300_mesh")
    n, nt, nnod, ntri, nnz = list(out)
    x, y, z = np.zeros(n), np.zeros(n), np.zeros(n)
    tetra = np.zeros(5 * nt, np.int32)
    rowptr = np.zeros(n + 1, np.int32)
    cols = np.zeros(nnz, np.int32)
    check(L.cathy_gb300_mesh(C.byref(mem.dem), iopt, out, _ptr(x, f64p), _ptr(y, f64p),
                             _ptr(z, f64p), _ptr(tetra, i32p), _ptr(rowptr, i32p),
                             _ptr(cols, i32p)), "cathy_gb300_mesh")
    return dict(n=n, nt=nt, nnod=nnod, ntri=ntri, x=x, y=y, z=z, tetra=tetra.reshape(nt, 5),
                rowptr=rowptr, cols=cols)


# ---------------------------------------------------------------------------
# Fortran drop-ins
# ---------------------------------------------------------------------------
def _ci(v):
    return C.byref(C.c_int32(int(v)))


def _cd(v):
    return C.byref(C.c_double(float(v)))


def symslv(topol, ja, coef1, tnoti, noddir, itmxcg=500, tolcg=1e-10, rmin=1.7e-100):
    """SYMSLV drop-in: IC(0)-PCG on the reference's symmetric upper CSR.
    Returns (pnew, niter, err, res, coef2)."""
    L = _lib.load()
    topol, ja, noddir = _i32(topol), _i32(ja), _i32(noddir)
    coef1, tnoti = _f64(coef1), _f64(tnoti)
    n, nterm = len(topol) - 1, len(ja)
    pnew, coef2 = np.zeros(n), np.zeros(nterm)
    niter = C.c_int32()
    err, res = C.c_double(), C.c_double()
    nd = noddir if len(noddir) else np.zeros(1, np.int32)
    check(L.cathy_gb300_symslv(_ci(6), _ci(n), _ci(nterm), _ci(len(noddir)), C.byref(niter),
                               _ci(itmxcg), _cd(tolcg), _cd(rmin), _ptr(nd, i32p),
                               _ptr(ja, i32p), _ptr(topol, i32p), _ptr(pnew, f64p),
                               _ptr(tnoti, f64p), _ptr(coef1, f64p), _ptr(coef2, f64p), None,
                               C.byref(err), C.byref(res)), "cathy_gb300_symslv")
    return pnew, niter.value, err.value, res.value, coef2


def nsyslv(topol, ja, coef1, tnoti, noddir, isolv=0, itmxcg=500, tolcg=1e-10,
           rmin=1.7e-100):
    """NSYSLV drop-in (ISOLV 0 ILU(0)-BiCGSTAB, -5 Jacobi-BiCGSTAB) on the
    reference's full CSR.  Returns (pnew, niter, err, res)."""
    L = _lib.load()
    topol, ja, noddir = _i32(topol), _i32(ja), _i32(noddir)
    coef1, tnoti = _f64(coef1), _f64(tnoti)
    n, nterm = len(topol) - 1, len(ja)
    ia = np.repeat(np.arange(1, n + 1, dtype=np.int32), np.diff(topol))
    pnew, coef2 = np.zeros(n), np.zeros(nterm)
    niter = C.c_int32()
    err, res = C.c_double(), C.c_double()
    nd = noddir if len(noddir) else np.zeros(1, np.int32)
    check(L.cathy_gb300_nsyslv(_ci(isolv), _ci(6), _ci(n), _ci(nterm), _ci(len(noddir)),
                               _ptr(nd, i32p), _ci(itmxcg), C.byref(niter), _ptr(ia, i32p),
                               _ptr(ja, i32p), _ptr(topol, i32p), _cd(tolcg), _cd(rmin),
                               _ptr(coef1, f64p), _ptr(coef2, f64p), _ptr(pnew, f64p),
                               _ptr(tnoti, f64p), C.byref(err), C.byref(res)),
          "cathy_gb300_nsyslv")
    return pnew, niter.value, err.value, res.value


def asspic(tetra, tetja, lmass, coef1, coef2, coef4, et1e, pel, permx, permy, permz,
           ckrwe, volu, volur, bi, ci, di, ntri, maxstr, etae=None):
    """ASSPIC drop-in (asspic.f:9): element assembly of the Picard stiffness
    (COEF1) and mass (COEF2, COEF4) arrays on the GPU.

    Arguments carry the reference's contents: ``tetra`` (nt, 5) and ``tetja``
    (nt, 4, 4) hold 1-based node ids / slot indices, ``tetja[e, l, k]`` being
    TETJA(K,L,IEL) (the Fortran array in memory order); ``lmass`` is LMASS
    (4, 4) in memory order; ``permx/permy/permz`` are PERMX(MAXSTR, NZONE)
    flattened in memory order; ``bi/ci/di`` are BI(4, NT) in memory order.
    The COEF arrays are accumulated (copies are returned)."""
    L = _lib.load()
    tetra, tetja = _i32(tetra).reshape(-1), _i32(tetja).reshape(-1)
    nt = len(tetra) // 5
    c1, c2, c4 = _f64(coef1).copy(), _f64(coef2).copy(), _f64(coef4).copy()
    nterm = len(c1)
    keep = [_f64(a).reshape(-1) for a in (lmass, et1e, pel, permx, permy, permz, ckrwe,
                                          volu, volur, bi, ci, di)]
    lm, a1, a2, px, py, pz, kr, vo, vr, b, c, d = keep
    et = _f64(etae) if etae is not None else np.zeros(nt)
    check(L.cathy_gb300_asspic(_ci(nt), _ci(ntri), _ptr(tetra, i32p), _ptr(tetja, i32p),
                               _ptr(lm, f64p), _ptr(c1, f64p), _ptr(c2, f64p), _ptr(c4, f64p),
                               _ptr(a1, f64p), _ptr(a2, f64p), _ptr(px, f64p), _ptr(py, f64p),
                               _ptr(pz, f64p), _ptr(kr, f64p), _ptr(et, f64p), _ptr(vo, f64p),
                               _ptr(vr, f64p), _ptr(b, f64p), _ptr(c, f64p), _ptr(d, f64p),
                               _ci(maxstr), _ci(nterm)), "cathy_gb300_asspic")
    return c1, c2, c4
