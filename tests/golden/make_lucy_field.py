"""Write tests/golden/full3d_tdust_phiavg.npz: the dust temperatures of the
full-3D benchmark model after the two Lucy set-up iterations of the
benchmark (2 x 2e6 packets, mixed form, on a GPU), averaged over azimuth.

Both arms of bench.py run their timed packets on this field (broadcast over
the azimuthal cells): the GPU arm, and the CPU restatement of the reference,
which cannot run the Lucy iterations itself in the time of a benchmark.  A
Lucy field gives the packet histories of the published run, whose peel-off
iteration follows five Lucy iterations; the analytic warm profile of the
tests makes the disk interior far hotter and its histories far longer.

Run from the repository root on a machine with a GPU:
    python tests/golden/make_lucy_field.py
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "full3d_tdust_phiavg.npz"
LUCY_PACKETS = 2_000_000


def main() -> None:
    from hochunk3d_gb300 import configs, hc3d
    from hochunk3d_gb300.build import build_library

    build_library()
    with tempfile.TemporaryDirectory() as td:
        m = hc3d.Model(configs.write_par(Path(td), "full3d"))
        ctx = hc3d.Context(hc3d.PREC_MIXED).load(m)
        for it in (1, 2):
            p = m.run_params(np=LUCY_PACKETS, iter=it, ipeel=0)
            ctx.zero()
            ctx.run(p)
            tdust, rel, _ = ctx.lucy_update(m.info.ltot, LUCY_PACKETS)
        ctx.close()
        nrg, ntg, npg, ndg = m.shape4
        has = m.densarr[:-1, :-1, :-1, :4] > 0
        t = tdust[:-1, :-1, :-1, :4]
        cnt = has.sum(axis=2)
        avg = np.where(cnt > 0, (t * has).sum(axis=2) / np.maximum(cnt, 1), t[:, :, 0, :])
        np.savez_compressed(OUT, tdust=avg.astype(np.float32), shape=np.array([nrg, ntg, npg, ndg]),
                            lucy_packets=LUCY_PACKETS, max_rel_change=rel)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


def field(model) -> np.ndarray:
    """The stored field broadcast over the azimuthal cells of model
    (nrg, ntg, npg, ndg), K/11605; raises when the model's grid differs."""
    z = np.load(OUT)
    nrg, ntg, npg, ndg = model.shape4
    if tuple(int(v) for v in z["shape"][:3]) != (nrg, ntg, npg):
        raise ValueError(f"{OUT.name} was made for grid {tuple(z['shape'])}, not {model.shape4}")
    td = np.full(model.shape4, 0.1 / 11605.0, order="F")
    avg = z["tdust"].astype(np.float64)  # (nrg-1, ntg-1, 4)
    td[:-1, :-1, :-1, :min(4, ndg)] = avg[:, :, None, :min(4, ndg)]
    return np.asfortranarray(td)


if __name__ == "__main__":
    main()
