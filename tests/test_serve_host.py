"""Host logic of the serving form (CPU): LRU admission under a byte budget with pinning,
the Poisson request stream, and the FIFO latency model."""
import numpy as np
import pytest

from vissatsatellitestereo_gb300.serve import ResidentStore, fifo_latencies, poisson_stream, state_bytes


def test_lru_admission_evicts_least_recent_unpinned():
    st = ResidentStore(100)
    for a, b in ((1, 40), (2, 30), (3, 20)):
        st.admit(b)
        st.put(a, f's{a}', b)
    assert st.used == 90
    assert st.get(1) == 's1'                 # 1 becomes most recent; LRU order 2, 3, 1
    ev = st.admit(25, pinned={2})
    assert ev == [3]                          # 2 is pinned, 3 is the oldest unpinned
    st.put(4, 's4', 25)
    assert st.used == 40 + 30 + 25 and 3 not in st and 2 in st
    assert st.evictions == 1
    ev = st.admit(35, pinned={2})
    assert ev == [1]                          # oldest first, only until 35 more fit
    assert st.used == 30 + 25


def test_admission_refuses_what_cannot_fit():
    st = ResidentStore(100)
    with pytest.raises(MemoryError):
        st.admit(101)
    st.admit(60)
    st.put(1, 'a', 60)
    with pytest.raises(MemoryError):
        st.admit(50, pinned={1})
    assert 1 in st and st.used == 60


def test_reput_replaces_bytes():
    st = ResidentStore(100)
    st.put(1, 'a', 10)
    st.put(1, 'b', 30)
    assert st.used == 30 and st.get(1) == 'b'


def test_poisson_stream_is_seeded_and_has_the_rate():
    a = poisson_stream(2000, 20.0, 400, seed=3)
    b = poisson_stream(2000, 20.0, 400, seed=3)
    assert [(r.aoi, r.arrival) for r in a] == [(r.aoi, r.arrival) for r in b]
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert abs(gaps.mean() - 0.05) < 0.005
    counts = np.bincount([r.aoi for r in a], minlength=400)
    assert counts.max() > 10 * np.median(counts[counts > 0])     # Zipf popularity


def test_fifo_latencies():
    lat = fifo_latencies([0.0, 0.1, 0.15], [0.2, 0.05, 0.01])
    assert np.allclose(lat, [0.2, 0.15, 0.11])


def test_state_bytes():
    from vissatsatellitestereo_gb300 import synth
    s = synth.AoiSpec(0, 3e5, 5e6, 0.5, 100, 50, 7, 2048, 1)
    assert state_bytes(s) == 4 * 100 * 50 * 7 + 8 * 14 * 7
