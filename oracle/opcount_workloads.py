"""Algorithmic FP64 operations per cell-update of the benchmark workloads
(measurement infrastructure: bench.py keeps the printed figures as constants).

Runs the oracle on the operation-counting scalar (hmr_opcount.cpp: add, sub,
mul, div, sqrt, fabs, fmin, fmax counted once each; the HLL part of HLLC-HLL
only on faces that select it) over EVERY patch of each workload with its own
initial state, and divides the summed operations of one RK stage by the summed
interior cells:

  python oracle/opcount_workloads.py            # all workloads, a few minutes on 8 cores
  python oracle/opcount_workloads.py --phases   # the default workload's count by sub-phase

  density_wave_256     2D single species, WCNS5-JS, one 256^2 patch
  shock_interface_1024 2D five-equation, WCNS6-LD, one 1024^2 patch
  blobs_512            3D single species, WCNS5-JS, 512 uneven cubic patches (side 16-64)
  shock_interface_3lv  3D five-equation, WCNS6-LD, the 3-level layout of uneven patches
"""
import ctypes
import multiprocessing
import os
import sys
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
LIB = os.path.join(HERE, "_build", "libhmr_opcount.so")


def _count(args):
    model, dim, nsp, scheme, gam, n, dx, Q = args
    L = ctypes.CDLL(LIB)
    L.hmro_count_ops.restype = ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    g = (ctypes.c_double * 8)(*(list(gam) + [1.4] * (8 - len(gam))))
    nn = (ctypes.c_int * 3)(*(list(n) + [1] * (3 - len(n))))
    d = (ctypes.c_double * 3)(*(list(dx) + [1.0] * (3 - len(dx))))
    per_cell = L.hmro_count_ops(model, dim, nsp, scheme, g, nn, d, Q.ctypes.data_as(dp))
    cells = int(np.prod(n))
    return per_cell * cells, cells


def density_wave_256():
    from hamers_gb300 import problems as P
    Q, dx, _ = P.density_wave_2d(256)
    yield (0, 2, 1, 0, [1.4], [256, 256], dx, Q)


def shock_interface_1024():
    from hamers_gb300 import problems as P
    Q, dx, _ = P.shock_interface_2d(N=1024, seed=1)
    yield (2, 2, 2, 1, [1.4, 1.67], [1024, 1024], dx, Q)


def blobs_512():
    # the layout and states bench.py times (blobs_patches_3d_device, evaluated on the CPU)
    from hamers_gb300 import problems as P
    for n, dx, Q in P.blobs_patches_3d_device(num_patches=512, device="cpu"):
        yield (0, 3, 1, 0, [1.4], n, dx, Q.numpy())


def shock_interface_3lv():
    import torch
    from hamers_gb300 import problems as P
    layout = P.amr_layout_3d(base=128, seed=4)
    amps, waves, phases = P.shock_interface_3d_modes(64, seed=4)
    a = torch.tensor(amps, dtype=torch.float64)
    finest = min(dx[0] for _, _, _, dx in layout)
    for _, lo, n, dx in layout:
        Q = P.shock_interface_3d_patch(lo, n, dx, a, waves, phases, finest).numpy()
        yield (2, 3, 2, 1, [1.4, 1.09], n, dx, Q)


PHASES = ["cell data", "sensor", "projection factors", "characteristic variables", "smoothness indicators",
          "weights + interpolation", "inverse projection", "bounds check", "Riemann (HLLC / HLLC-HLL)",
          "flux formula", "advective source", "stage update"]


def phases(model, dim, nsp, scheme, gam, n, dx, Q):
    """Algorithmic FP64 operations per cell-update of one patch, by sub-phase."""
    L = ctypes.CDLL(LIB)
    L.hmro_count_ops.restype = ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    g = (ctypes.c_double * 8)(*(list(gam) + [1.4] * (8 - len(gam))))
    nn = (ctypes.c_int * 3)(*(list(n) + [1] * (3 - len(n))))
    d = (ctypes.c_double * 3)(*(list(dx) + [1.0] * (3 - len(dx))))
    total = L.hmro_count_ops(model, dim, nsp, scheme, g, nn, d, Q.ctypes.data_as(dp))
    out = (ctypes.c_double * len(PHASES))()
    L.hmro_count_phases(nn, dim, out)
    return total, list(out)


def phase_table():
    """The default workload (2D five-equation WCNS6-LD, counted at 256^2 of its problem)."""
    from hamers_gb300 import problems as P
    Q, dx, _ = P.shock_interface_2d(N=256, seed=1)
    total, ph = phases(2, 2, 2, 1, [1.4, 1.67], [256, 256], dx, Q)
    print("| sub-phase | FP64 ops per cell-update | share |")
    print("|---|---|---|")
    for name, v in zip(PHASES, ph):
        print(f"| {name} | {v:.1f} | {100 * v / total:.1f} % |")
    print(f"| total | {total:.1f} | |")


def main():
    if sys.argv[1:] == ["--phases"]:
        phase_table()
        return
    if not os.path.exists(LIB):
        import subprocess
        subprocess.check_call(["make", "-s", "-C", HERE])
    names = sys.argv[1:] or ["density_wave_256", "shock_interface_1024", "blobs_512", "shock_interface_3lv"]
    ctx = multiprocessing.get_context("spawn")
    with ProcessPoolExecutor(max_workers=os.cpu_count() or 1, mp_context=ctx) as ex:
        for name in names:
            res = list(ex.map(_count, globals()[name](), chunksize=1))
            ops = sum(r[0] for r in res)
            cells = sum(r[1] for r in res)
            print(f"{name}: {ops / cells:.1f} FP64 ops per cell-update ({len(res)} patches, {cells} cells)",
                  flush=True)


if __name__ == "__main__":
    main()
