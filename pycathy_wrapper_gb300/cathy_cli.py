"""``./cathy`` replacement: run the CATHY project in the current directory.

pyCATHY compiles CATHY into ``./cathy`` inside the project folder and runs it
there (pyCATHY/cathy_tools.py:669, ``run_processor``; the IPRT1 = 3 mesh run
at :729).  A launcher named ``cathy`` in the project folder that executes

    python -m pycathy_wrapper_gb300.cathy_cli

takes its place: it reads ``input/`` and ``prepro/`` of the current
directory, runs the subsurface solver on the GPU (or, with IPRT1 = 3, only
writes the mesh files, on the host) and writes the ``output/`` files
pyCATHY reads.  The exit status is 0 when the run reached TMAX.
"""
from __future__ import annotations

import argparse
import os
import sys


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="cathy", description=__doc__.splitlines()[0])
    ap.add_argument("project", nargs="?", default=os.getcwd(),
                    help="project folder (default: the current directory)")
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1],
                    help="0: FP64 throughout; 1: FP32 Krylov inside FP64 Picard (default)")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    from .pycathy import run_project
    res = run_project(os.path.abspath(args.project), precision=args.precision,
                      device=args.device)
    if "mesh" in res:
        m = res["mesh"]
        print(f"cathy: mesh written (NNOD {m['nnod']}, N {m['n']}, NT {m['nt']})")
        return 0
    status = {0: "running", 1: "finished", 2: "failed"}.get(res["status"], "?")
    print(f"cathy: {status} at TIME {res['time']:.6g} after {res['steps']} steps")
    return 0 if res["status"] == 1 else 1


if __name__ == "__main__":
    sys.exit(main())
