"""The allocation-free solve entry point (cathy_gb300_nsyslv_noalloc).

Callers such as a Fortran driver whose device memory belongs to a host
framework's pool may not call cudaMalloc while they run.  For them the
library exports a variant of the NSYSLV ISOLV=-5 solve that works on device
buffers the caller already owns and keeps its own workspace in a fixed
device array.  These tests call it through the C ABI and check it against
the allocating entry point cathy_gb300_nsyslv on the same system, twice in a
row (the second call reuses the workspace the first one left behind).

The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden_case


def _system():
    """The soil3d golden case's first Picard matrix in the reference's full
    CSR storage, with the 1e-9*RMAX Dirichlet penalty a Fortran caller
    passes to NSYSLV."""
    import oracle as O
    import scipy.sparse as sp
    case = load_golden_case("soil3d")
    o = O.Oracle(case)
    c1, tn, xt5, dm = o.picard_system()
    om = o.mesh()
    n = o.n
    rows = np.repeat(np.arange(n), np.diff(om["topol"]))
    U = sp.csr_matrix((c1, (rows, om["ja"] - 1)), shape=(n, n))
    A = (U + U.T - sp.diags(U.diagonal())).tolil()
    noddir = (np.nonzero(dm)[0] + 1).astype(np.int32)
    for d in noddir - 1:
        A[d, d] = 1.7e91
    A = A.tocsr()
    A.sort_indices()
    topol = (A.indptr + 1).astype(np.int32)
    ja = (A.indices + 1).astype(np.int32)
    return topol, ja, A.data.astype(np.float64), np.asarray(tn, np.float64), noddir


def _ci(v):
    return C.byref(C.c_int32(int(v)))


def _cd(v):
    return C.byref(C.c_double(float(v)))


def test_noalloc_rejects_systems_beyond_its_workspace():
    from pycathy_wrapper_gb300 import _lib
    L = _lib.load()
    niter, err, res = C.c_int32(), C.c_double(), C.c_double()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.cathy_gb300_nsyslv_noalloc(_ci(131072 + 1), _ci(0), None, _ci(10), C.byref(niter),
                                      dummy, dummy, _cd(1e-10), dummy, dummy, dummy,
                                      C.byref(err), C.byref(res), None)
    assert rc == _lib.EINVAL


@pytest.mark.gpu
def test_noalloc_matches_allocating_nsyslv_twice():
    import torch
    from pycathy_wrapper_gb300 import _lib
    from pycathy_wrapper_gb300.api import nsyslv
    L = _lib.load()
    topol, ja, vals, tn, noddir = _system()
    n = len(topol) - 1
    assert n <= 131072
    x_ref, n_ref, e_ref, r_ref = nsyslv(topol, ja, vals, tn, noddir, isolv=-5,
                                        itmxcg=500, tolcg=1e-10)
    dev = torch.device("cuda:0")
    t_topol = torch.from_numpy(topol).to(dev)
    t_ja = torch.from_numpy(ja).to(dev)
    t_vals = torch.from_numpy(vals).to(dev)
    t_tn = torch.from_numpy(tn).to(dev)
    t_nod = torch.from_numpy(noddir).to(dev)
    torch.cuda.synchronize()
    scale = np.max(np.abs(x_ref))
    # the second call runs on a stream of its own: the entry point must
    # launch on the stream it is given
    side = torch.cuda.Stream(device=dev)
    outs = [torch.full((n,), float("nan"), dtype=torch.float64, device=dev) for _ in range(2)]
    torch.cuda.synchronize()
    for call in range(2):
        t_x = outs[call]
        stream = None if call == 0 else C.c_void_p(side.cuda_stream)
        free_before = torch.cuda.mem_get_info(dev)[0]
        niter, err, res = C.c_int32(), C.c_double(), C.c_double()
        rc = L.cathy_gb300_nsyslv_noalloc(
            _ci(n), _ci(len(noddir)), C.c_void_p(t_nod.data_ptr()), _ci(500), C.byref(niter),
            C.c_void_p(t_ja.data_ptr()), C.c_void_p(t_topol.data_ptr()), _cd(1e-10),
            C.c_void_p(t_vals.data_ptr()), C.c_void_p(t_x.data_ptr()),
            C.c_void_p(t_tn.data_ptr()), C.byref(err), C.byref(res), stream)
        assert rc == _lib.OK, (call, rc)
        if call == 1:
            # after the first call (which loads the library's device code and
            # its fixed workspace) a call takes no device memory
            side.synchronize()
            assert torch.cuda.mem_get_info(dev)[0] == free_before
        torch.cuda.synchronize()
        x = t_x.cpu().numpy()
        # same tolerance as the NSYSLV drop-in's own parity test
        assert np.all(np.isfinite(x)), call
        assert np.max(np.abs(x - x_ref)) <= 1e-7 * scale, (call, np.max(np.abs(x - x_ref)))
        assert abs(niter.value - n_ref) <= 1, (call, niter.value, n_ref)
        assert err.value <= 1e-10
        assert res.value <= 10.0 * r_ref + 1e-14, (call, res.value, r_ref)
