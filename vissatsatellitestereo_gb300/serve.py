"""Serving form: a stream of AOI fusion requests over HBM-resident AOI state.

A request asks for the fused DSM of one AOI of a catalog (aggregate_2p5d.py:65-81 over
the AOI's per-view DSMs of produce_dsm.py:46-58).  The server keeps, per AOI, its camera
set (the perspective fits of camera_approx.py:150-204) and its partial DSMs (one float32
DSM per view) resident in HBM under an admission budget, evicting the least recently used
AOIs that no batch on the device still needs.  A request for a resident AOI costs one
fusion; a miss first brings the AOI's height maps to the device when they are held in
host memory (the request's inputs: one copy per view on the batch's stream), rasterises
all of its views (one persistent tile launch for all misses of the batch, straight into
the resident stacks) and fits its cameras.

Continuous batching with overlap on the device: every iteration takes all requests that
have arrived (up to ``max_batch``) as one batch and issues its work -- misses, fits,
fusions and the copy of each fused DSM into pinned host memory -- on one of ``slots``
CUDA streams, without waiting for it.  The loop then polls the batches' completion events,
finishes the requests of completed batches (their latency includes the copy back), and
admits newly arrived requests as soon as a slot is free, so batches run concurrently on
the GPU.  A batch that needs an AOI another in-flight batch is still materialising waits
for it on the device (an event), not on the host.  The result of a request does not depend
on what it is batched or overlapped with (every kernel writes only its own AOI's buffers).
"""
import collections
import time
from dataclasses import dataclass

import numpy as np
import torch

from .aggregate_2p5d import fuse_dsms
from .batch import AoiBatch, AoiGrid, MapAffine, MapView, upload_map


@dataclass
class Request:
    rid: int
    aoi: int
    arrival: float            # seconds after the stream starts
    done: float = None
    hit: bool = None
    batch: int = None


def poisson_stream(n_requests, rate, n_aois, seed, zipf_s=1.0):
    """Requests with exponential inter-arrival gaps (Poisson arrivals at ``rate`` per second)
    over AOIs drawn with Zipf(``zipf_s``) popularity (a seeded permutation of the catalog)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n_requests)
    arrivals = np.cumsum(gaps)
    ranks = np.arange(1, n_aois + 1, dtype=np.float64)
    p = ranks ** -zipf_s
    p /= p.sum()
    order = rng.permutation(n_aois)
    picks = order[rng.choice(n_aois, size=n_requests, p=p)]
    return [Request(i, int(a), float(t)) for i, (a, t) in enumerate(zip(picks, arrivals))]


class ResidentStore:
    """Least-recently-used map AOI -> resident state under a byte budget (host bookkeeping;
    the states hold device tensors, freed when evicted)."""

    def __init__(self, budget_bytes):
        self.budget = int(budget_bytes)
        self.used = 0
        self.items = collections.OrderedDict()      # aoi -> (state, nbytes)
        self.hits = self.misses = self.evictions = 0

    def get(self, aoi):
        item = self.items.get(aoi)
        if item is None:
            return None
        self.items.move_to_end(aoi)
        return item[0]

    def admit(self, nbytes, pinned=()):
        """Evict least recently used AOIs outside ``pinned`` until ``nbytes`` more fit.
        Returns the evicted AOIs; raises MemoryError when they cannot be made to fit."""
        nbytes = int(nbytes)
        if nbytes > self.budget:
            raise MemoryError(f'AOI state of {nbytes} bytes exceeds the budget of {self.budget}')
        evicted = []
        for aoi in list(self.items):
            if self.used + nbytes <= self.budget:
                break
            if aoi in pinned:
                continue
            _, b = self.items.pop(aoi)
            self.used -= b
            self.evictions += 1
            evicted.append(aoi)
        if self.used + nbytes > self.budget:
            raise MemoryError('the AOIs pinned by the batch leave no room')
        return evicted

    def put(self, aoi, state, nbytes):
        if aoi in self.items:
            self.used -= self.items.pop(aoi)[1]
        self.items[aoi] = (state, int(nbytes))
        self.used += int(nbytes)

    def __contains__(self, aoi):
        return aoi in self.items


def state_bytes(spec):
    """Resident bytes of one AOI: a float32 DSM per view plus its camera parameters."""
    return 4 * spec.cells * spec.n_views + 8 * 14 * spec.n_views


def pool_view_source(specs, pool, affines):
    """View source over a height-map pool (on the device, or in pinned host memory, from
    where a miss copies the windows it needs): view k of AOI a reads pool map
    (first view index of a + k) mod P, window [:image, :image]."""
    first = np.concatenate([[0], np.cumsum([s.n_views for s in specs])]).tolist()
    P = pool.shape[0]

    def views_of(a):
        s = specs[a]
        return [(pool[(first[a] + v) % P], s.image, s.image, aff) for v, aff in enumerate(affines[a])]
    return views_of


class _InFlight:
    """A batch whose work is on the device: its requests, host copies, completion event and
    everything that must stay alive until the event fires."""

    def __init__(self, index, batch, stream, outs, hosts, event, keep, aois):
        self.index, self.batch, self.stream = index, batch, stream
        self.outs, self.hosts, self.event, self.keep, self.aois = outs, hosts, event, keep, aois


class FusionServer:
    def __init__(self, specs, view_source, metas=None, budget_bytes=150 << 30, max_batch=64, tile=64,
                 blocks_per_sm=4, fit_grid=(200, 20), slots=3):
        """specs: the AOI catalog (``synth.AoiSpec``: grid and view count); view_source(a):
        the AOI's views as (CUDA float32 heights, width, height, fixed-point affine dict);
        metas: per AOI the views' RPC meta_dicts (None: no camera fits); slots: batches that
        may be on the device at once (one CUDA stream each)."""
        self.specs = list(specs)
        self.view_source = view_source
        self.metas = metas
        self.store = ResidentStore(budget_bytes)
        self.max_batch = int(max_batch)
        self.tile = tile
        self.blocks_per_sm = blocks_per_sm
        self.fit_grid = fit_grid
        self.slots = max(1, int(slots))
        self.streams = [torch.cuda.Stream() for _ in range(self.slots)]
        self.inflight = []
        self.max_inflight = 0
        self.pixels = 0               # height-map pixels rasterised
        self.cell_views = 0           # per-view DSM cells produced
        self.fused_cell_views = 0     # cell-views read by fusions
        self.fit_points = 0
        self.batches = 0
        self.h2d_bytes = 0            # height maps copied from host memory for misses

    # ---- misses -----------------------------------------------------------------------
    def _views(self, a, stack):
        """The AOI's views as device maps: maps held in host memory (the request's inputs)
        are copied to the device on the current stream first."""
        out = []
        for v, (h, w, hh, aff) in enumerate(self.view_source(a)):
            if not h.is_cuda:
                h = upload_map(h, w, hh)
                self.h2d_bytes += 4 * w * hh
            out.append(MapView(h, w, hh, MapAffine(**aff), dsm=stack[v]))
        return out

    def _rasterise(self, aois, stacks):
        grids = [AoiGrid(self.specs[a].xoff, self.specs[a].yoff, self.specs[a].res, self.specs[a].res,
                         self.specs[a].xsize, self.specs[a].ysize) for a in aois]
        plan = AoiBatch(grids, [self._views(a, stacks[a]) for a in aois], tile=self.tile)
        plan.run(None, blocks_per_sm=self.blocks_per_sm)
        self.pixels += plan.pixels
        self.cell_views += plan.view_cells
        return plan

    def _fit(self, a):
        from . import synth
        from .camera_approx import approx_perspective_enu
        ms = self.metas[a]
        g = synth.rpc_sample_grid_torch(ms[0], self.fit_grid[0], self.fit_grid[1], 'cuda')
        params, err, status = approx_perspective_enu(ms, g['lat'], g['lon'], g['alt'], g['x'], g['y'], g['z'])
        self.fit_points += len(ms) * g['lat'].numel()
        return params, err, status

    def _materialise(self, misses, pinned):
        """Admit, rasterise (all missing AOIs' views in one launch, straight into their
        resident stacks) and fit the missing AOIs on the current stream.  Returns the plans,
        which must outlive the work."""
        stacks, plans, states = {}, [], []
        for a in misses:
            s = self.specs[a]
            self.store.admit(state_bytes(s), pinned)
            stack = torch.empty((s.n_views, s.ysize, s.xsize), dtype=torch.float32, device='cuda')
            stacks[a] = stack
            cams = self._fit(a) if self.metas is not None else None
            state = {'stack': stack, 'cameras': cams, 'stream': torch.cuda.current_stream(), 'ready': None}
            states.append(state)
            self.store.put(a, state, state_bytes(s))
        plans.append(self._rasterise(misses, stacks))
        ready = torch.cuda.Event()
        ready.record()
        for st in states:
            st['ready'] = ready
        return plans

    # ---- requests ---------------------------------------------------------------------
    def _pinned(self, batch):
        pinned = {r.aoi for r in batch}
        for f in self.inflight:
            pinned |= f.aois
        return pinned

    def issue(self, batch):
        """Issue one batch's work on the current stream without waiting for it; returns the
        fused DSMs (device tensors, valid once the stream reaches them) and the objects that
        must stay alive until then."""
        self.batches += 1
        pinned = self._pinned(batch)
        st = torch.cuda.current_stream()
        misses = []
        for r in batch:
            hit = r.aoi in self.store and r.aoi not in misses
            r.hit = hit
            if hit:
                self.store.hits += 1
            else:
                self.store.misses += 1
                if r.aoi not in misses:
                    misses.append(r.aoi)
        plans = self._materialise(misses, pinned) if misses else []
        outs = []
        for r in batch:
            state = self.store.get(r.aoi)
            stack = state['stack']
            if state['stream'] != st:
                # built on another stream: order after it on the device, and tell the
                # allocator that this stream uses the stack too
                if state['ready'] is not None:
                    st.wait_event(state['ready'])
                stack.record_stream(st)
            outs.append(fuse_dsms(stack, median_blur=True, layout='vhw'))
            self.fused_cell_views += stack.numel()
        return outs, plans

    def process(self, batch):
        """Serve one batch of requests on the current stream; returns their fused DSMs
        (device tensors; synchronise the stream before reading them on the host)."""
        outs, plans = self.issue(batch)
        torch.cuda.current_stream().synchronize()
        for p in plans:
            p.close()
        return outs

    def _retire(self, f, t_done, outputs, keep_outputs, on_batch):
        for r, h in zip(f.batch, f.hosts):
            r.done = t_done
            r.batch = f.index
            if keep_outputs:
                outputs[r.rid] = h
        if on_batch:
            on_batch(f.batch, f.hosts)
        for p in f.keep:
            p.close()

    def run_stream(self, requests, realtime=True, keep_outputs=False, on_batch=None):
        """Serve ``requests`` (sorted by arrival).  In real time, a request cannot be taken
        before its arrival time.  Each batch (all arrived requests, up to max_batch) goes to
        a free slot's stream; completed batches are found by polling their events.  A
        request is done when its fused DSM is in host memory.  Returns the latency
        statistics (and the host DSMs by request id with ``keep_outputs``)."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        outputs = {}
        t0 = time.perf_counter()
        busy, busy_since = 0.0, None
        next_stream = 0
        while pending or self.inflight:
            now = time.perf_counter() - t0
            for f in [f for f in self.inflight if f.event.query()]:
                self.inflight.remove(f)
                self._retire(f, time.perf_counter() - t0, outputs, keep_outputs, on_batch)
            if not self.inflight and busy_since is not None:
                busy += time.perf_counter() - t0 - busy_since
                busy_since = None
            now = time.perf_counter() - t0
            if pending and len(self.inflight) < self.slots and (not realtime or pending[0].arrival <= now):
                batch = []
                while pending and len(batch) < self.max_batch and (not realtime or pending[0].arrival <= now):
                    batch.append(pending.popleft())
                stream = self.streams[next_stream % self.slots]
                next_stream += 1
                if busy_since is None:
                    busy_since = now
                with torch.cuda.stream(stream):
                    outs, plans = self.issue(batch)
                    hosts = []
                    for o in outs:
                        h = torch.empty(o.shape, dtype=o.dtype, pin_memory=True)
                        h.copy_(o, non_blocking=True)
                        hosts.append(h)
                    ev = torch.cuda.Event()
                    ev.record(stream)
                self.inflight.append(_InFlight(self.batches, batch, stream, outs, hosts, ev, plans,
                                               {r.aoi for r in batch}))
                self.max_inflight = max(self.max_inflight, len(self.inflight))
                continue
            if self.inflight:
                time.sleep(5e-5)
            elif pending and realtime:
                time.sleep(min(max(pending[0].arrival - now, 0.0), 0.05))
        if busy_since is not None:
            busy += time.perf_counter() - t0 - busy_since
        wall = time.perf_counter() - t0
        lat = np.array([r.done - r.arrival for r in requests])
        hits = np.array([bool(r.hit) for r in requests])
        stats = {
            'requests': len(requests), 'wall_s': round(wall, 3), 'gpu_busy_s': round(busy, 3),
            'p50_latency_ms': round(float(np.percentile(lat, 50)) * 1e3, 3),
            'p99_latency_ms': round(float(np.percentile(lat, 99)) * 1e3, 3),
            'mean_latency_ms': round(float(lat.mean()) * 1e3, 3),
            'p50_hit_latency_ms': round(float(np.percentile(lat[hits], 50)) * 1e3, 3) if hits.any() else None,
            'p99_miss_latency_ms': round(float(np.percentile(lat[~hits], 99)) * 1e3, 3) if (~hits).any() else None,
            'hit_rate': round(float(hits.mean()), 4), 'evictions': self.store.evictions, 'batches': self.batches,
            'slots': self.slots, 'max_batches_in_flight': self.max_inflight,
            'resident_gb_end': round(self.store.used / 2 ** 30, 2),
            'pixels_per_s_busy': self.pixels / busy if busy else None,
            'dsm_cells_per_s_busy': self.cell_views / busy if busy else None,
            'fused_cell_views_per_s_busy': self.fused_cell_views / busy if busy else None,
            'rpc_fit_pts_per_s_busy': self.fit_points / busy if busy else None,
            'h2d_map_gb': round(self.h2d_bytes / 1e9, 2),
            'latency': 'arrival to the fused DSM in host memory (pinned), polled completion events',
            'busy': 'wall time during which at least one batch was on the device',
        }
        return (stats, outputs) if keep_outputs else stats


def fifo_latencies(arrivals, service):
    """Latencies of a single FIFO server with the given arrival and service times."""
    t, out = 0.0, []
    for a, s in zip(arrivals, service):
        t = max(t, a) + s
        out.append(t - a)
    return np.array(out)
