"""Time the reference's NumPy step against the oracle port on the same
sample, one core each -- MEASUREMENT INFRASTRUCTURE ONLY.

The reference is pure Python and exists only where its sources are
present, so the CPU baseline that travels with the benchmark is the port
(oracle/sdader_oracle.py).  This script measures how far the port's speed
is from the reference's, for the record:

    OMP_NUM_THREADS=1 python oracle/calibrate_port.py /path/to/reference 64 3

(four-quadrant problem, p=3, FV update with limiting, HLLC, N x N cells,
one warm-up step and K timed steps each; prints seconds per step and the
port / reference ratio).
"""
from __future__ import annotations

import os
import sys
import time
import warnings

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main(ref_root, n, steps):
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    warnings.simplefilter("ignore")
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import bench
    from sdader_simulator import SDADER_Simulator as Reference
    kw = bench.workload_kwargs("quadrant512", n)
    s = Reference(use_cupy=False, verbose=False, **kw)
    s.init_sim()
    s.compute_dt()
    s.perform_update()
    t0 = time.perf_counter()
    for _ in range(steps):
        s.compute_dt()
        s.perform_update()
    t_ref = (time.perf_counter() - t0) / steps
    _, el = bench._cpu_worker(("quadrant512", n, steps, 1))
    t_port = el / steps
    print(f"{n}x{n}: reference {t_ref:.3f} s/step, port {t_port:.3f} s/step, port/reference {t_port / t_ref:.3f}")


if __name__ == "__main__":
    main(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 64, int(sys.argv[3]) if len(sys.argv) > 3 else 3)
