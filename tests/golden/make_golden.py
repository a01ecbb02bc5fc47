"""Generate the golden trace fixtures of the parity tests.

For the small models ``tiny`` (axisymmetric) and ``tiny3d`` (azimuthal walls
and a fractal envelope), both with the warm temperature profile of
tests/helpers.py, this records with the CPU oracle:

* the single-packet traces of 32 packets fed splitmix64 uniforms (the
  bit-exact cell-index criterion): kind, ir, it, ip, iface, tsum, x, y, z;
* a 2000-packet run on the Philox streams: escape/peel counts, absorption
  counts and the event counters.

Run from the repository root:  python tests/golden/make_golden.py
The oracle is the project's CPU restatement of the reference (the reference
itself cannot be built here), so these fixtures pin the GPU library and the
oracle against regressions, not the oracle against the reference.
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from hochunk3d_gb300.build import build_library, build_oracle  # noqa: E402
from tests.helpers import make_model, splitmix_uniforms  # noqa: E402

NPKT, NU, MAXREC, NRUN = 32, 20000, 2048, 2000


def main() -> None:
    build_library()
    build_oracle()
    import oracle.oracle as O

    out = Path(__file__).resolve().parent
    with tempfile.TemporaryDirectory() as td:
        for name in ("tiny", "tiny3d"):
            m = make_model(Path(td) / name, name, warm=True)
            p = m.run_params(np=NPKT, iter=3, ipeel=1)
            U = splitmix_uniforms(NPKT, NU, seed=1000 + len(name))
            recs, nrec, exhausted = [], [], []
            for k in range(NPKT):
                r, ex, _ = O.trace(m, p, k, U[k], max_rec=MAXREC)
                recs.append(r)
                nrec.append(len(r))
                exhausted.append(ex)
            allrec = np.concatenate(recs)
            pr = m.run_params(np=NRUN, iter=3, ipeel=1)
            res = O.run(m, pr)
            np.savez_compressed(
                out / f"trace_{name}.npz",
                seed=np.int64(1000 + len(name)), nu=np.int64(NU), nrec=np.array(nrec, np.int32),
                exhausted=np.array(exhausted, bool),
                kind=allrec["kind"], ir=allrec["ir"], it=allrec["it"], ip=allrec["ip"], iface=allrec["iface"],
                tsum=allrec["tsum"], x=allrec["x"], y=allrec["y"], z=allrec["z"],
                run_np=np.int64(NRUN), run_nums=res["nums"].sum(axis=(1, 2, 3)), run_numt=res["numt"].sum(axis=(1, 2)),
                run_nabs=res["nabs"].sum(axis=(0, 1, 2)), run_counters=res["counters"],
            )
            print(name, "records", len(allrec), "exhausted", sum(exhausted), "counters", res["counters"][:15])


if __name__ == "__main__":
    main()
