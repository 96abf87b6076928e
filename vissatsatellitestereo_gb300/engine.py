"""Many-AOI execution: waves of AOIs sized to an HBM budget, batched or per-view launches,
CUDA-graph capture and a small autotuner for the batched launches' work shapes.

An ``AoiSetEngine`` owns the device data of a set of AOIs (per-view FP32 height maps as
windows of a resident map pool, fixed-point pixel -> UTM maps, DSM grids) and runs the
reference's per-AOI chain -- per-view DSMs (produce_dsm.py:46-58) and their fusion
(aggregate_2p5d.py:65-81) -- for all of them.  AOIs are grouped into consecutive waves
whose per-view DSMs (4 bytes per cell-view) fit ``budget_bytes``; each wave is one
``AoiBatch`` plan.  ``step('batched')`` issues per wave one rasterisation launch over all
its views' DSM tiles, then the per-AOI fusions; ``step('per_view')`` issues the same kernel
one view at a time (the per-view form).  Fused DSMs of all AOIs land in one resident
buffer.
"""
import torch

from .batch import AoiBatch, AoiGrid, MapAffine, MapView


class AoiSetEngine:
    def __init__(self, specs, pool, affines, budget_bytes=96 << 30, tile=64, blocks_per_sm=4):
        """specs: AOI specs (``synth.AoiSpec``); pool: (P, S, S) CUDA float32 map pool (view
        k of the set reads pool map k % P, window [:image, :image]); affines: per AOI, the
        per-view fixed-point maps (dicts)."""
        self.specs = list(specs)
        self.pool = pool
        self.affines = affines
        self.budget = int(budget_bytes)
        self.tile = int(tile)
        self.blocks_per_sm = int(blocks_per_sm)
        self._build()

    # ---- plans ------------------------------------------------------------------------
    def _views_of(self, a, k0):
        s = self.specs[a]
        P = self.pool.shape[0]
        out = []
        for v, aff in enumerate(self.affines[a]):
            m = self.pool[(k0 + v) % P]
            out.append(MapView(m, s.image, s.image, MapAffine(**aff)))
        return out

    def _build(self):
        self.waves, self.wave_aois = [], []
        cur, cur_bytes, k = [], 0, 0
        groups = []
        for a, s in enumerate(self.specs):
            need = 4 * s.cells * s.n_views
            if cur and cur_bytes + need > self.budget:
                groups.append(cur)
                cur, cur_bytes = [], 0
            cur.append((a, k))
            cur_bytes += need
            k += s.n_views
        if cur:
            groups.append(cur)
        for g in groups:
            grids = [AoiGrid(self.specs[a].xoff, self.specs[a].yoff, self.specs[a].res, self.specs[a].res,
                             self.specs[a].xsize, self.specs[a].ysize) for a, _ in g]
            views = [self._views_of(a, k0) for a, k0 in g]
            self.waves.append(AoiBatch(grids, views, tile=self.tile))
            self.wave_aois.append([a for a, _ in g])
        self.view_dsm = torch.empty(max(w.view_cells for w in self.waves), dtype=torch.float32, device='cuda')
        self.scratch = torch.empty(max(w.scratch_bytes for w in self.waves), dtype=torch.uint8, device='cuda')
        self.fused_off = [0]
        for w in self.waves:
            self.fused_off.append(self.fused_off[-1] + w.fused_cells)
        self.fused = torch.empty(self.fused_off[-1], dtype=torch.float32, device='cuda')
        self.pixels = sum(w.pixels for w in self.waves)
        self.cell_views = sum(w.view_cells for w in self.waves)
        self.cells = self.fused_off[-1]
        self.n_views = sum(w.n_views for w in self.waves)
        self.graph = None

    def close(self):
        for w in self.waves:
            w.close()
        self.graph = None

    # ---- execution ----------------------------------------------------------------------
    def run_wave(self, i, mode='batched'):
        w = self.waves[i]
        fused = self.fused[self.fused_off[i]:self.fused_off[i + 1]]
        if mode == 'batched':
            w.run(self.view_dsm, blocks_per_sm=self.blocks_per_sm)
        else:
            for v in range(w.n_views):
                w.run(self.view_dsm, views=(v, v + 1), blocks_per_sm=self.blocks_per_sm)
        w.fuse(self.view_dsm, fused, self.scratch)

    def step(self, mode='batched'):
        if mode == 'graph':
            if self.graph is None:
                self.capture()
            self.graph.replay()
            return
        for i in range(len(self.waves)):
            self.run_wave(i, mode)

    def capture(self):
        """Capture one batched step (all waves) in a CUDA graph."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.step('batched')          # warm: lazy attribute setup happens outside capture
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step('batched')
        torch.cuda.synchronize()
        self.graph = g

    def fused_dsm(self, a):
        """The fused (H, W) DSM of AOI a (valid after a step)."""
        for i, aois in enumerate(self.wave_aois):
            if a in aois:
                j = aois.index(a)
                buf = self.fused[self.fused_off[i]:self.fused_off[i + 1]]
                return self.waves[i].fused_dsm(buf, j)
        raise IndexError(a)

    # ---- tuning -------------------------------------------------------------------------
    def time_step(self, mode='batched', reps=1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            self.step(mode)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    def autotune(self, tiles=(32, 64), blocks=(2, 3, 4, 6, 8), wave=0):
        """Pick the DSM tile edge and the CTAs per SM (capped by what fits) by timing the
        batched rasterisation of one wave for every pair; re-plans all waves with the winner.
        Returns the timings."""
        w0 = self.waves[wave]
        grids = w0.grids
        views = w0.views
        timings = {}
        for t in tiles:
            b = AoiBatch(grids, views, tile=t)
            for bl in blocks:
                b.run(self.view_dsm, blocks_per_sm=bl)       # warm
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record()
                b.run(self.view_dsm, blocks_per_sm=bl)
                e1.record()
                torch.cuda.synchronize()
                timings[(t, bl)] = e0.elapsed_time(e1) / 1e3
            b.close()
        (t, bl) = min(timings, key=timings.get)
        if t != self.tile or bl != self.blocks_per_sm:
            self.close()
            self.tile, self.blocks_per_sm = t, bl
            self._build()
        return {f'tile{k[0]}_blocks{k[1]}': round(v * 1e3, 3) for k, v in timings.items()}


class AoiCameraFits:
    """Perspective fits of every view of a set of AOIs (camera_approx.py:150-204 per AOI):
    each AOI's views project its shared lat/lon/alt grid; one fused-pipeline call per AOI.
    Cameras, grids and outputs are resident, so ``step`` only launches kernels."""

    def __init__(self, specs, metas, n_xy=200, n_z=20, mode='fast'):
        from . import _lib, synth
        from .rpc_model import MODES
        self._lib = _lib
        self.mode = MODES[mode]
        self.items = []
        ws = 0
        for s, ms in zip(specs, metas):
            cams = torch.from_numpy(_lib.camera_array(ms)).cuda()
            g = synth.rpc_sample_grid_torch(ms[0], n_xy, n_z, 'cuda')
            V, n = len(ms), g['lat'].numel()
            params = torch.empty((V, _lib.VS_CAMERA_PARAMS), dtype=torch.float64, device='cuda')
            err = torch.empty((V, _lib.VS_ERROR_STATS), dtype=torch.float64, device='cuda')
            status = torch.empty((V,), dtype=torch.int32, device='cuda')
            self.items.append((cams, g, V, n, params, err, status))
            ws = max(ws, _lib.lib().vs_camera_approx_workspace_size(V, n))
        self.ws = torch.empty(max(ws, 256), dtype=torch.uint8, device='cuda')
        self.points = sum(V * n for _, _, V, n, _, _, _ in self.items)

    def step(self):
        from ._dev import stream_handle
        st = stream_handle()
        for cams, g, V, n, params, err, status in self.items:
            self._lib.call('vs_camera_approx_perspective', cams.data_ptr(), V, g['lat'].data_ptr(),
                           g['lon'].data_ptr(), g['alt'].data_ptr(), g['x'].data_ptr(), g['y'].data_ptr(),
                           g['z'].data_ptr(), n, 0, self.mode, params.data_ptr(), err.data_ptr(), status.data_ptr(),
                           self.ws.data_ptr(), self.ws.numel(), st)

    def status_ok(self):
        return all(bool((st == 0).all()) for *_, st in self.items)
