"""CPU oracle for the VisSat geometry path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy/scipy, the reference algorithms of the four
routines the GPU library replaces.  It exists to check the CUDA path and to time the
CPU baseline; the product never imports it.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU legs of ``bench.py`` may use it, and only as the checker / the timed CPU
baseline.

Pinning: ``rpc`` and ``dlt`` are checked bit-for-bit (rpc) and to rounding (dlt)
against golden vectors produced by importing the reference's own
``lib/rpc_model.py``, ``lib/solve_perspective.py`` and ``lib/check_error.py``
(``tests/golden/make_golden.py``).  ``raster`` and ``fuse`` are checked against golden
vectors produced by executing the reference's own source lines
(``lib/proj_to_grid.py:42-79`` with a restated ``numpy_groupies`` 0.9.9 ``nanmax``,
and ``aggregate_2p5d.py:68-78``).  The third-party arithmetic on the path, which is not
installed here, is restated from its published source: ``blur`` from OpenCV 4.0.0's
``medianBlur_SortNet`` (ksize 3, float32: the sorting network and its scalar/SSE
compare-exchange, which decide what NaN does), ``quat`` from pyquaternion 0.9.5's
``Quaternion._from_matrix``, ``geo`` from pymap3d 1.7.15's ``enu2geodetic`` chain and
PROJ 6.2's ``utm`` (pyproj 2.4).

Modules:
  rpc     -- apply_poly / apply_rfm / projection        (lib/rpc_model.py:40-168)
  dlt     -- solve_perspective / factorize / error        (lib/solve_perspective.py, lib/check_error.py)
  raster  -- proj_to_grid                                  (lib/proj_to_grid.py:41-81)
  blur    -- cv2.medianBlur(float32, 3)                   (produce_dsm.py:58, aggregate_2p5d.py:81)
  fuse    -- per-cell MAD-filtered mean of per-view DSMs   (aggregate_2p5d.py:65-81)
  quat    -- rotation matrix -> quaternion                 (camera_approx.py:178, pyquaternion 0.9.5)
"""
