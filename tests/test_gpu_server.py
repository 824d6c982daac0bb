"""The serving runtime (aqsg_server_*): requests admitted by arrival time and
HBM onto concurrent lanes give the same outcomes as the same circuit run
alone through the direct API (State.apply / Program.run, then
State.sample_seeded), whether they run alone on the server or in a mix;
admission never holds more register bytes than the slab."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from afquantumsim_gb300 import circuits

pytestmark = pytest.mark.gpu

SHOTS = 256


def requests(count, seed, n_range=(6, 18), depth_range=(2, 8)):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        d = int(rng.integers(depth_range[0], depth_range[1] + 1))
        fuse = int(rng.choice([0, 0, 3, 4]))
        out.append(dict(n=n, ops=circuits.brickwork(n, d, seed=1000 + i), fuse=fuse,
                        seed=int(rng.integers(1 << 40))))
    return out


def direct(ctx, r):
    st = aq.State(ctx, r["n"])
    st.set_basis(0)
    if r["fuse"]:
        p = aq.Program(r["n"], r["ops"], max_qubits=r["fuse"])
        p.run(st, aq.EXEC_TILED)
        p.free()
    else:
        st.apply(r["ops"], aq.EXEC_TILED)
    out = st.sample_seeded(r["seed"], SHOTS)
    st.free()
    return out


def run_server(reqs, arrivals, budget, lanes, max_qubits=18):
    srv = aq.Server(0, aq.C64, budget, lanes, max_qubits, SHOTS)
    tickets = [srv.submit(r["n"], r["ops"], SHOTS, r["seed"], a, r["fuse"]) for r, a in zip(reqs, arrivals)]
    srv.start()
    srv.wait_idle(300)
    done = {d["ticket"]: d for d in srv.poll(len(reqs) + 8)}
    stats = srv.stats()
    srv.close()
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    return [done[t] for t in tickets], stats


def test_server_alone_and_in_mix_match_direct(gpu_ctx):
    reqs = requests(24, seed=21)
    want = [direct(gpu_ctx, r) for r in reqs]
    # each request alone on a fresh server
    for r, w in zip(reqs[:6], want[:6]):
        (d,), _ = run_server([r], [0.0], 1 << 22, 1)
        assert d["status"] == 0
        np.testing.assert_array_equal(d["outcomes"], w)
    # all of them as a Poisson stream over 4 lanes
    arr = np.cumsum(np.random.default_rng(5).exponential(0.002, size=len(reqs)))
    got, stats = run_server(reqs, list(arr), 1 << 24, 4)
    for r, d, w in zip(reqs, got, want):
        assert d["status"] == 0 and d["n"] == r["n"]
        assert d["admit_s"] >= d["arrival_s"] - 1e-9 and d["done_s"] >= d["admit_s"]
        np.testing.assert_array_equal(d["outcomes"], w)
    assert stats["peak_bytes"] <= stats["slab_bytes"]
    assert stats["launches"] > 0


def test_server_admission_bounded_by_slab(gpu_ctx):
    # slab of two 18-qubit registers; 18-qubit requests queue behind each
    # other while small ones pass them
    reqs = requests(16, seed=8, n_range=(14, 18), depth_range=(2, 4))
    got, stats = run_server(reqs, [0.0] * len(reqs), 2 * 8 << 18, 6)
    assert stats["slab_bytes"] == 2 * 8 << 18
    assert stats["peak_bytes"] <= stats["slab_bytes"]
    assert all(d["status"] == 0 for d in got)
    want = [direct(gpu_ctx, r) for r in reqs]
    for d, w in zip(got, want):
        np.testing.assert_array_equal(d["outcomes"], w)


def test_server_rejects_bad_requests():
    srv = aq.Server(0, aq.C64, 1 << 22, 2, 12, 64)
    with pytest.raises(aq.OutOfRange):
        srv.submit(13, [aq.H(0)], 8)
    with pytest.raises(aq.OutOfRange):
        srv.submit(4, [aq.H(0)], 65)
    with pytest.raises(aq.OutOfRange, match="Cannot add gate at the given qubit position"):
        srv.submit(4, [aq.X(4)], 8)
    with pytest.raises(aq.InvalidArgument):
        srv.submit(4, [aq.H(0)], 8, fuse_qubits=6)
    srv.close()
    with pytest.raises(aq.InvalidArgument):
        aq.Server(0, aq.C64, 1 << 10, 2, 12, 64)  # budget below one 12-qubit register


def test_server_c128_zero_shots_and_late_submit(gpu_ctx):
    """complex128 server; a request with no shots completes; requests
    submitted after start with arrival -1 are admitted at once."""
    srv = aq.Server(0, aq.C128, 1 << 24, 2, 16, 64)
    srv.start()
    reqs = requests(4, seed=31, n_range=(6, 16), depth_range=(2, 4))
    tickets = [srv.submit(r["n"], r["ops"], 64 if k else 0, r["seed"], -1.0, 0) for k, r in enumerate(reqs)]
    srv.wait_idle(120)
    done = {d["ticket"]: d for d in srv.poll(16)}
    assert set(done) == set(tickets) and all(d["status"] == 0 for d in done.values())
    assert done[tickets[0]]["outcomes"].size == 0
    for k in range(1, 4):  # same draws as the direct complex128 path
        r = reqs[k]
        with aq.State(gpu_ctx, r["n"], aq.C128) as st:
            st.set_basis(0)
            st.apply(r["ops"], aq.EXEC_TILED)
            want = st.sample_seeded(r["seed"], 64)
        np.testing.assert_array_equal(done[tickets[k]]["outcomes"], want)
    srv.close()


def test_server_close_with_queued_requests():
    """Requests still queued (arrival far in the future) are dropped on
    close; the call returns promptly."""
    import time
    srv = aq.Server(0, aq.C64, 1 << 22, 1, 12, 8)
    for k in range(5):
        srv.submit(10, circuits.brickwork(10, 2, seed=k), 8, k, 3600.0, 0)
    srv.start()
    t0 = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t0 < 5.0


def test_server_requests_as_text(gpu_ctx):
    """A request submitted as circuit text gives the outcomes of the same ops
    submitted directly."""
    reqs = requests(3, seed=44, n_range=(8, 14), depth_range=(2, 4))
    srv = aq.Server(0, aq.C64, 1 << 22, 2, 14, SHOTS)
    t_ops = [srv.submit(r["n"], r["ops"], SHOTS, r["seed"], -1.0, r["fuse"]) for r in reqs]
    t_txt = [srv.submit_text(aq.circuit_to_text(r["n"], r["ops"]), SHOTS, r["seed"], -1.0, r["fuse"])
             for r in reqs]
    srv.start()
    srv.wait_idle(120)
    done = {d["ticket"]: d for d in srv.poll(16)}
    srv.close()
    for a, b in zip(t_ops, t_txt):
        assert done[a]["status"] == 0 and done[b]["status"] == 0
        np.testing.assert_array_equal(done[a]["outcomes"], done[b]["outcomes"])
