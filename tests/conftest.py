import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


def load_golden_case(key):
    """Rebuild a Case from the fixture written by tests/golden/make_golden.py."""
    from pycathy_wrapper_gb300.inputs import BC, Case, Dem, Parm, Soil
    z = np.load(os.path.join(GOLDEN, f"{key}_case.npz"))
    meta = json.loads(str(z["meta"]))
    dem = Dem(dem=z["dem"], delta_x=meta["delta_x"], delta_y=meta["delta_y"],
              zratio=z["zratio"], base=meta["base"], ivert=meta["ivert"],
              zone=z["zone"].astype(np.int32), west=meta["west"],
              south=meta["south"], factor=meta["factor"])
    soil = Soil(**{k: z["soil_" + k] for k in ("permx", "permy", "permz", "elstor",
                                               "poros", "vgn", "vgrmc", "vgpsat")},
                pmin=meta["pmin"], scf=meta["scf"], kslope=meta["kslope"],
                tolksl=meta["tolksl"],
                feddes=z["soil_feddes"] if "soil_feddes" in z else None,
                root_map=z["soil_root_map"] if "soil_root_map" in z else None)
    parm = Parm(**meta["parm"])
    bc = BC(atmtim=z["atmtim"], atminp=z["atminp"], hspatm=meta["hspatm"],
            ieto=meta["ieto"], indp=meta["indp"], wtposition=meta["wtposition"],
            pinit=z["pinit"] if "pinit" in z else None)
    return Case(dem, soil, parm, bc, name=key)


def golden_json():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
