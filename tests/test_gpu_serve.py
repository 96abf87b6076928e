"""Serving form on the GPU: a request's fused DSM is the same alone and in a batch, after
evictions, and equal to the oracle's (bit-exact)."""
import numpy as np
import pytest
import torch

from conftest import same_bits
from oracle import maps as omaps

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def catalog():
    from vissatsatellitestereo_gb300 import synth
    specs, maps, affines = synth.small_aoi_case()
    dev = [[torch.from_numpy(m).cuda() for m in ms] for ms in maps]

    def views_of(a):
        return [(h, h.shape[1], h.shape[0], aff) for h, aff in zip(dev[a], affines[a])]
    ref = []
    for s, ms, afs in zip(specs, maps, affines):
        g = {'xoff': s.xoff, 'yoff': s.yoff, 'xres': s.res, 'yres': s.res, 'xsize': s.xsize, 'ysize': s.ysize}
        ref.append(omaps.fused_dsm([omaps.view_dsm(m, a, g) for m, a in zip(ms, afs)]))
    return specs, views_of, ref


def serve(specs, views_of, aois, batched, budget=1 << 30):
    from vissatsatellitestereo_gb300.serve import FusionServer, Request
    srv = FusionServer(specs, views_of, budget_bytes=budget)
    reqs = [Request(i, a, 0.0) for i, a in enumerate(aois)]
    stats, outs = srv.run_stream(reqs, realtime=False, keep_outputs=True) if batched else (None, {})
    if not batched:
        for r in reqs:
            outs[r.rid] = srv.process([r])[0]
        torch.cuda.synchronize()
    return srv, reqs, {k: v.cpu().numpy() for k, v in outs.items()}


def test_alone_and_in_the_mix_are_identical_and_match_the_oracle(catalog):
    specs, views_of, ref = catalog
    aois = [0, 1, 2, 0, 2, 1, 1]
    _, reqs_a, alone = serve(specs, views_of, aois, batched=False)
    srv, reqs_b, mixed = serve(specs, views_of, aois, batched=True)
    assert srv.batches == 1                       # every request arrived: one batch
    for r in reqs_b:
        assert same_bits(alone[r.rid], mixed[r.rid])
        assert same_bits(mixed[r.rid], ref[r.aoi])
    assert [r.hit for r in reqs_a] == [False, False, False, True, True, True, True]


def test_eviction_and_recompute_give_the_same_bits(catalog):
    from vissatsatellitestereo_gb300.serve import state_bytes
    specs, views_of, ref = catalog
    budget = max(state_bytes(s) for s in specs)    # room for one AOI at a time
    srv, reqs, outs = serve(specs, views_of, [0, 1, 0, 2, 0], batched=False, budget=budget)
    assert srv.store.evictions >= 2
    seen, recomputed = set(), False
    for r in reqs:                                 # an AOI served before was rebuilt after eviction
        recomputed |= r.aoi in seen and not r.hit
        seen.add(r.aoi)
    assert recomputed
    for r in reqs:
        assert same_bits(outs[r.rid], ref[r.aoi])


def test_overlapping_batches_match_alone_and_the_oracle(catalog):
    """Batches of one request each on three streams: every batch starts with a bounded GPU
    delay (torch.cuda._sleep, ~10 ms), so the host issues the next batches while earlier
    ones are still on the device -- with hits on AOIs that another in-flight batch is still
    building.  Every fused DSM (copied back to the host) equals the one served alone and the
    oracle's."""
    from vissatsatellitestereo_gb300.serve import FusionServer, Request
    specs, views_of, ref = catalog
    aois = [0, 1, 0, 2, 1, 2, 0, 1]
    _, reqs_a, alone = serve(specs, views_of, aois, batched=False)
    srv = FusionServer(specs, views_of, budget_bytes=1 << 30, max_batch=1, slots=3)
    issue = srv.issue

    def delayed_issue(batch):
        torch.cuda._sleep(20_000_000)           # a fixed number of GPU clock cycles
        return issue(batch)
    srv.issue = delayed_issue
    reqs = [Request(i, a, 0.0) for i, a in enumerate(aois)]
    stats, outs = srv.run_stream(reqs, realtime=False, keep_outputs=True)
    assert stats['max_batches_in_flight'] >= 2 and srv.batches == len(aois)
    assert any(r.hit for r in reqs)
    for r in reqs:
        got = outs[r.rid].numpy()
        assert same_bits(got, alone[r.rid])
        assert same_bits(got, ref[r.aoi])


def test_host_held_maps_give_the_same_bits(catalog):
    """Requests whose height maps live in pinned host memory (copied to the device by the
    misses, windows of a larger map) serve the same fused DSMs as device-held maps."""
    from vissatsatellitestereo_gb300 import synth
    from vissatsatellitestereo_gb300.batch import upload_map
    specs, views_of, ref = catalog
    _, maps, affines = synth.small_aoi_case()
    host = []
    for ms in maps:
        hs = []
        for m in ms:
            big = torch.full((m.shape[0] + 3, m.shape[1] + 5), 7.0, dtype=torch.float32).pin_memory()
            big[:m.shape[0], :m.shape[1]] = torch.from_numpy(m)
            hs.append(big)
        host.append(hs)

    def host_views(a):
        return [(h, m.shape[1], m.shape[0], aff) for h, m, aff in zip(host[a], maps[a], affines[a])]
    up = upload_map(host[0][0], maps[0][0].shape[1], maps[0][0].shape[0])
    torch.cuda.synchronize()
    assert same_bits(up.cpu().numpy(), maps[0][0])
    aois = [0, 1, 2, 0, 2]
    srv, reqs, outs = serve(specs, host_views, aois, batched=True)
    assert srv.h2d_bytes == sum(4 * m.size for a in (0, 1, 2) for m in maps[a])
    for r in reqs:
        assert same_bits(outs[r.rid], ref[r.aoi])
