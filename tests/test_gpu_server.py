"""Continuous-batching server: results are the same alone and in a mix, memory
admission, cancellation and host-side fault injection (no GPU fault)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _requests(seed, n, dev="cuda"):
    """Mixed graded lattices (blend mode) and CSG scenes of assorted sizes."""
    from gpucadforam_gb300.mesher import Lattice, make_frame, primitives_to_device

    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        edge = int(np.exp(rng.uniform(np.log(24), np.log(96))))
        shape = (edge, edge, edge)
        if rng.random() < 0.7:
            C = 4
            nc = C ** 3
            lat = Lattice.from_numpy(1, (C, C, C), rng.uniform(8, 24, nc).astype(np.float32),
                                     rng.uniform(-0.7, 0.7, 3 * nc).astype(np.float32),
                                     rng.uniform(-0.5, 0.5, nc).astype(np.float32),
                                     rng.choice(np.array([0, 1, 5], np.uint8), nc), device=dev)
            reqs.append(("lattice", lat, shape))
        else:
            k = int(rng.integers(8, 33))
            prims = []
            for j in range(k):
                c = rng.uniform(0, 1, 3)
                kind = int(rng.integers(0, 3))
                op = 1 if j >= k - 3 else 0
                if kind == 0:
                    prims.append(dict(kind=0, op=op, center=c, p=[rng.uniform(0.05, 0.2), 0.0]))
                elif kind == 1:
                    prims.append(dict(kind=1, op=op, center=c, v3=(0, 0, 1), p=[rng.uniform(0.03, 0.12), 0.0,
                                                                                   rng.uniform(0.1, 0.3)]))
                else:
                    prims.append(dict(kind=2, op=op, center=c, p=list(rng.uniform(0.05, 0.25, 3))))
            h = np.float32(1.0 / (edge - 1))
            reqs.append(("csg", (primitives_to_device(prims, dev), k, make_frame((0, 0, 0), (h, h, h))), shape))
    return reqs


def _submit(srv, req, tag):
    kind, payload, shape = req
    if kind == "lattice":
        return srv.submit_lattice(payload, shape, 0.0, tag)
    prims, k, frame = payload
    return srv.submit_csg(prims, k, frame, shape, 0.0, tag)


def _alone(req):
    """The same request through the single-grid public calls."""
    from gpucadforam_gb300.mesher import Context

    ctx = Context(0)
    kind, payload, shape = req
    field = ctx.lattice_field(payload, shape) if kind == "lattice" else ctx.csg_field(payload[0], payload[1],
                                                                                      payload[2], shape)
    pos, norm, cnt = ctx.mesh_field(field, 0.0)
    out = pos.cpu().numpy(), norm.cpu().numpy(), cnt.total_verts
    ctx.close()
    return out


def test_results_identical_alone_and_in_the_mix():
    from gpucadforam_gb300.mesher import Server

    reqs = _requests(0xD4A + 5, 24)
    srv = Server(lanes=4, device_pool_bytes=4 << 30, host_pool_bytes=2 << 30)
    tickets = {}
    for i, r in enumerate(reqs):
        rc, t = _submit(srv, r, i)
        assert rc == 0
        tickets[t] = i
    got = srv.drain(tickets)
    assert len(got) == len(reqs)
    lanes = set()
    for t, (res, pos, norm) in got.items():
        assert res.status == 0
        lanes.add(res.lane)
        apos, anorm, n = _alone(reqs[tickets[t]])
        assert res.total_verts == n
        assert pos.tobytes() == apos[:n].tobytes() and norm.tobytes() == anorm[:n].tobytes()
    assert len(lanes) > 1  # the mix really ran on several lanes
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["device_pool_used"] == 0
    srv.close()


def test_over_budget_requests_are_rejected():
    from gpucadforam_gb300.mesher import Lattice, Server

    srv = Server(lanes=2, device_pool_bytes=64 << 20, host_pool_bytes=64 << 20)
    lat = Lattice.from_numpy(0, (1, 1, 1), np.array([16.0], np.float32))
    rc, _ = srv.submit_lattice(lat, (400, 400, 400))  # 256 MB field > 64 MB pool
    assert rc == 8  # GCM_ERR_REJECTED at submission
    # field fits, mesh does not: rejected after counting
    rc, t = srv.submit_lattice(lat, (200, 200, 200))
    assert rc == 0
    (res, _, _), = srv.drain([t]).values()
    assert res.status == 8
    assert srv.stats()["device_pool_used"] == 0
    srv.close()


def test_cancel_pending_request():
    from gpucadforam_gb300.mesher import Server

    reqs = _requests(3, 6)
    srv = Server(lanes=1, device_pool_bytes=2 << 30, host_pool_bytes=1 << 30, fault_flags=2, fault_param=200)
    ts = [_submit(srv, r, i)[1] for i, r in enumerate(reqs)]
    assert srv.cancel(ts[-1]) == 0
    got = srv.drain(ts)
    assert got[ts[-1]][0].status == 9  # GCM_ERR_CANCELLED
    assert all(got[t][0].status == 0 for t in ts[:-1])
    srv.close()


def test_injected_pool_failures_are_retried():
    from gpucadforam_gb300.mesher import Server

    reqs = _requests(5, 8)
    srv = Server(lanes=2, device_pool_bytes=2 << 30, host_pool_bytes=1 << 30, fault_flags=1, fault_param=2)
    ts = [_submit(srv, r, i)[1] for i, r in enumerate(reqs)]
    got = srv.drain(ts)
    assert all(got[t][0].status == 0 for t in ts)
    assert srv.stats()["pool_faults"] > 0
    srv.close()
    # every reservation failing: the requests fail cleanly with GCM_ERR_OUT_OF_MEMORY
    srv = Server(lanes=2, device_pool_bytes=2 << 30, host_pool_bytes=1 << 30, fault_flags=1, fault_param=1)
    ts = [_submit(srv, r, i)[1] for i, r in enumerate(reqs[:3])]
    got = srv.drain(ts)
    assert all(got[t][0].status == 5 for t in ts)
    srv.close()


def test_dead_lane_requeues_and_slow_lane_does_not_block():
    from gpucadforam_gb300.mesher import Server

    reqs = _requests(7, 10)
    srv = Server(lanes=3, device_pool_bytes=2 << 30, host_pool_bytes=1 << 30, fault_flags=4)
    ts = [_submit(srv, r, i)[1] for i, r in enumerate(reqs)]
    got = srv.drain(ts)
    assert all(got[t][0].status == 0 for t in ts)
    st = srv.stats()
    assert st["lanes_alive"] == 2 and st["requeued"] >= 1
    assert all(got[t][0].lane != 0 for t in ts)
    srv.close()
    srv = Server(lanes=3, device_pool_bytes=2 << 30, host_pool_bytes=1 << 30, fault_flags=2, fault_param=300)
    ts = [_submit(srv, r, i)[1] for i, r in enumerate(reqs)]
    got = srv.drain(ts)
    assert all(got[t][0].status == 0 for t in ts)
    assert sum(1 for t in ts if got[t][0].lane != 0) >= len(ts) - 2
    srv.close()
