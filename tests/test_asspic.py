"""ASSPIC (asspic.f:9-54): the oracle's restatement against an independent
numpy assembly (CPU), and the GPU drop-in cathy_gb300_asspic against the
oracle on the golden weill case (GPU): the drop-in gathers each slot's
contributions in the reference's element order with separately rounded
products and sums, so it must agree bit for bit, call after call.
"""
import numpy as np
import pytest

from conftest import load_golden_case


def _inputs():
    import oracle as O
    case = load_golden_case("weill")
    o = O.Oracle(case)
    o.picard_system()  # brings CKRWE/ET1E to the first iteration's state
    a = o.asspic_inputs()
    rng = np.random.default_rng(7)
    nterm = o.nterm
    # nonzero starting arrays: ASSPIC accumulates into the caller's arrays
    c0 = [rng.standard_normal(nterm) * 1e-6 for _ in range(3)]
    return o, a, c0


def _numpy_asspic(a, c0):
    """COEF1/COEF2/COEF4 from the element formulas, vectorised (sum order
    differs from the reference: compared with a tolerance)."""
    tetra, tetja = a["tetra"], a["tetja"].reshape(-1, 4, 4)  # [e, l, k]
    nt = len(tetra)
    ntri, maxstr = a["ntri"], a["maxstr"]
    iel = np.arange(1, nt + 1)
    istr = 1 + iel // (ntri * 3)
    istr = np.where(iel % (ntri * 3) == 0, istr - 1, istr)
    idx = (istr - 1) + maxstr * (tetra[:, 4] - 1)
    vk = a["volur"] * a["ckrwe"]
    b, c, d = (a[k].reshape(nt, 4) for k in ("bi", "ci", "di"))
    lm = a["lmass"].reshape(4, 4)  # [l, k]
    c1, c2, c4 = (x.copy() for x in c0)
    for k in range(4):
        for l in range(k, 4):
            ind = tetja[:, l, k] - 1
            v1 = vk * (a["permx"][idx] * b[:, k] * b[:, l] + a["permy"][idx] * c[:, k] * c[:, l]
                       + a["permz"][idx] * d[:, k] * d[:, l])
            np.add.at(c1, ind, v1)
            np.add.at(c2, ind, a["volu"] * a["et1e"] * lm[l, k])
            np.add.at(c4, ind, a["volu"] * a["pel"] * lm[l, k])
    return c1, c2, c4


def _args(a):
    return dict(tetra=a["tetra"], tetja=a["tetja"], lmass=a["lmass"], et1e=a["et1e"],
                pel=a["pel"], permx=a["permx"], permy=a["permy"], permz=a["permz"],
                ckrwe=a["ckrwe"], volu=a["volu"], volur=a["volur"], bi=a["bi"], ci=a["ci"],
                di=a["di"], ntri=a["ntri"], maxstr=a["maxstr"])


def test_oracle_asspic_matches_numpy_assembly():
    import oracle as O
    o, a, c0 = _inputs()
    got = O.asspic(coef1=c0[0], coef2=c0[1], coef4=c0[2], **_args(a))
    ref = _numpy_asspic(a, c0)
    for g, r in zip(got, ref):
        scale = np.max(np.abs(r))
        assert np.max(np.abs(g - r)) <= 1e-13 * scale


@pytest.mark.gpu
def test_asspic_dropin_matches_oracle_bit_for_bit():
    import oracle as O
    from pycathy_wrapper_gb300.api import asspic
    o, a, c0 = _inputs()
    ref = O.asspic(coef1=c0[0], coef2=c0[1], coef4=c0[2], **_args(a))
    first = asspic(coef1=c0[0], coef2=c0[1], coef4=c0[2], **_args(a))
    again = asspic(coef1=c0[0], coef2=c0[1], coef4=c0[2], **_args(a))
    for r, g1, g2 in zip(ref, first, again):
        np.testing.assert_array_equal(g1, g2)  # deterministic
        np.testing.assert_array_equal(g1, r)   # the reference's sums, bit for bit


@pytest.mark.gpu
def test_asspic_dropin_rejects_bad_tetja():
    from pycathy_wrapper_gb300.api import asspic
    o, a, c0 = _inputs()
    bad = a["tetja"].copy()
    bad[5] = o.nterm + 1
    args = _args(a)
    args["tetja"] = bad
    from pycathy_wrapper_gb300._lib import CathyError
    with pytest.raises(CathyError):
        asspic(coef1=c0[0], coef2=c0[1], coef4=c0[2], **args)
