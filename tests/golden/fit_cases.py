"""Fit problems pinned at the benchmarked sizes, shared by ``make_golden.py`` (which fits
them with the reference's own code) and the tests (which regenerate the grids)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from vissatsatellitestereo_gb300 import synth  # noqa: E402


def fit_cases():
    """The fit problems pinned at the benchmarked sizes: (name, metas, n_xy, n_z, shared).

    * ``cfg1_<size>``: one camera each of 2048, 4096 and 8192 px over its own 200x200x20
      grid (the per-view fit of the 50-view AOI workload);
    * ``cfg0``: one 2048 px camera over a 101x101x21 grid (the single-camera workload);
    * ``shared``: three cameras (2048, 4096, 8192 px) sharing one normalisation and one
      200x200x20 grid, the reference's own call pattern (camera_approx.py:158-176 projects
      one lat/lon/alt grid through every camera).
    """
    seed = synth.BASE_SEED
    cases = []
    for i, size in enumerate((2048, 4096, 8192)):
        cases.append((f'cfg1_{size}', [synth.make_rpc_meta(seed + 1000 + i, size, size)], 200, 20, False))
    cases.append(('cfg0', [synth.make_rpc_meta(seed + 1100, 2048, 2048)], 101, 21, False))
    base = synth.make_rpc_meta(seed + 1200, 4096, 4096)
    shared = []
    for i, size in enumerate((2048, 4096, 8192)):
        m = synth.make_rpc_meta(seed + 1201 + i, size, size)
        for k in ('latOff', 'latScale', 'lonOff', 'lonScale', 'altOff', 'altScale'):
            m['rpc'][k] = base['rpc'][k]
        shared.append(m)
    cases.append(('shared', shared, 200, 20, True))
    return cases
