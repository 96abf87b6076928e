"""vissat-gb300: the VisSat satellite-stereo geometry path on GB300 (sm_103a).

Drop-in replacements for the reference's four data-parallel routines, each backed by
hand-written CUDA kernels behind the C ABI of ``include/vissat_gb300.h``:

  RPCModel.projection         (lib/rpc_model.py)          -> rpc_model.RPCModel
  solve_perspective           (lib/solve_perspective.py)   -> solve_perspective
  check_perspective_error     (lib/check_error.py)         -> check_error
  approx_perspective_enu loop (camera_approx.py)           -> camera_approx
  proj_to_grid                (lib/proj_to_grid.py)        -> proj_to_grid
  produce_dsm_from_points     (produce_dsm.py)             -> produce_dsm
  run_fuse fusion block       (aggregate_2p5d.py)          -> aggregate_2p5d.fuse_dsms
"""
__version__ = '0.1.0'
