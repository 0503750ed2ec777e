"""Continuous-batching request loop (aeros_gb300/serve.py)."""
import io
import json

import numpy as np
import pytest

SMALL_GRIDS = ((32, 16, 16), (40, 24, 24), (48, 24, 16))


def test_requests_are_seeded_poisson():
    from aeros_gb300 import serve
    a = serve.make_requests(400, rate=2.0, seed=7)
    b = serve.make_requests(400, rate=2.0, seed=7)
    assert [(r.arrival, r.grid, r.freq, r.re) for r in a] == [(r.arrival, r.grid, r.freq, r.re) for r in b]
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert (gaps > 0).all()
    assert 0.4 < gaps.mean() < 0.6            # mean gap 1 / rate
    assert 0.7 < gaps.std() / gaps.mean() < 1.3   # exponential: coefficient of variation 1
    assert all(50.0 <= r.re <= 1000.0 for r in a)
    assert {r.grid for r in a} == set(serve.SERVE_GRIDS)
    assert all(serve.SERVE_FREQS[0] <= r.freq <= serve.SERVE_FREQS[1] for r in a)
    tris = [20 * r.freq * r.freq for r in a]
    assert min(tris) < 40000 and max(tris) > 450000   # 20k .. 500k triangles


def test_footprint_estimate_orders_requests():
    from aeros_gb300 import serve
    small = serve.Request(0, 0.0, (48, 48, 48), 32, 100.0, 1)
    big = serve.Request(1, 0.0, (256, 128, 128), 158, 100.0, 2)
    assert serve.footprint_estimate(small) < serve.footprint_estimate(big)
    assert serve.footprint_estimate(big, "fp32") > serve.footprint_estimate(big, "fp16")


def _reqs(serve, n):
    return serve.make_requests(n, rate=50.0, seed=11, grids=SMALL_GRIDS, freqs=(4, 8))


@pytest.mark.gpu
def test_result_alone_equals_result_in_mix():
    """A request served alone and among five others: the same Cd, step count,
    and bitwise the same final populations."""
    from aeros_gb300 import serve
    reqs = _reqs(serve, 6)
    kept = {}

    def keep(res, solver):
        kept[res.rid] = solver.populations()

    srv = serve.Server(check_every=200, max_steps=1000, chunk=100, tol=1e-3)
    mix = srv.run(reqs, realtime=False, on_retire=keep)
    mix_pop = dict(kept)
    kept.clear()
    target = reqs[3]
    alone = srv.run([target], realtime=False, on_retire=keep)
    a = alone["results"][0]
    m = [r for r in mix["results"] if r.rid == target.rid][0]
    assert (a.steps, a.converged) == (m.steps, m.converged)
    assert a.cd == m.cd and np.isfinite(a.cd)
    assert np.array_equal(kept[target.rid], mix_pop[target.rid])
    s = mix["summary"]
    assert s["requests"] == 6 and s["p50_s"] <= s["p95_s"] <= s["p99_s"]


@pytest.mark.gpu
def test_admission_respects_slots_and_budget():
    from aeros_gb300 import serve
    reqs = _reqs(serve, 5)

    def max_overlap(results):
        ev = sorted([(r.admitted, 1) for r in results] + [(r.finished, -1) for r in results])
        cur = best = 0
        for _, d in ev:
            cur += d
            best = max(best, cur)
        return best

    two = serve.Server(slots=2, check_every=200, max_steps=400, chunk=100).run(reqs, realtime=False)
    assert max_overlap(two["results"]) <= 2 and two["summary"]["requests"] == 5
    tight = serve.Server(budget_bytes=serve.footprint_estimate(reqs[0]) + 1, check_every=200, max_steps=400,
                         chunk=100).run(reqs, realtime=False)
    assert max_overlap(tight["results"]) == 1 and tight["summary"]["requests"] == 5
    assert all(r.steps == 400 or r.converged for r in tight["results"])


def test_geodesic_meshes_are_closed_and_outward():
    """The serving meshes (class-I geodesic spheres, 20 n^2 triangles): every
    edge is shared by exactly two triangles in opposite directions (closed,
    as the voxelizer's parity test needs) and every face points outward."""
    from aeros_gb300 import geometry
    for n in (1, 3, 32):
        v, c = geometry.geodesic_unit(n)
        assert len(c) == 20 * n * n and len(v) == 10 * n * n + 2
        e = np.concatenate([c[:, [0, 1]], c[:, [1, 2]], c[:, [2, 0]]])
        fwd = set((e[:, 0] * len(v) + e[:, 1]).tolist())
        assert len(fwd) == len(e) and fwd == set((e[:, 1] * len(v) + e[:, 0]).tolist())
        t = v[c]
        nrm = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
        assert (np.einsum("ij,ij->i", nrm, t.mean(axis=1)) > 0).all()


@pytest.mark.gpu
def test_sequential_baseline_runs_each_request_to_its_end():
    """The one-at-a-time baseline steps every request until its own Cd
    converges or the cap: measured, with the serving loop's rule."""
    from aeros_gb300 import serve
    reqs = _reqs(serve, 3)
    seq = serve.sequential_plain(reqs, check_every=200, tol=1e-3, max_steps=600)
    assert len(seq["per_request"]) == 3 and seq["wall_s"] > 0
    for p in seq["per_request"]:
        assert p["steps"] % 200 == 0 and 0 < p["steps"] <= 600
        assert p["converged"] or p["steps"] == 600


def test_solve_json_line():
    """Per-solve line: status, Cd trace, latency and the request's own rate
    over its time in the batch (cells x steps / (finished - started))."""
    from aeros_gb300 import serve
    r = serve.Result(3, 1.0, 1.5, 11.0, 2000, 0.61, True, 1_000_000, 20480, 123, started=2.0,
                     cd_trace=[(1000, 0.6), (2000, 0.61)], storage="fp16")
    d = json.loads(r.json_line())
    assert d["status"] == "converged" and d["steps"] == 2000 and d["cd_trace"] == [[1000, 0.6], [2000, 0.61]]
    assert d["latency_s"] == 10.0 and d["queued_s"] == 0.5
    assert d["mlups"] == round(1e6 * 2000 / 9.0 / 1e6, 1)
    assert d["gbs"] == round(r.mlups * 101 / 1e3, 1)
    c = serve.Result(4, 0.0, 0.2, 0.2, 0, float("nan"), False, 8, 20, 0, cancelled=True)
    d = json.loads(c.json_line())
    assert d["status"] == "cancelled" and d["cd"] is None and d["mlups"] == 0.0 and d["cd_trace"] == []
    s = serve.summarize([r, c], 10.0, 0)
    assert s["requests"] == 1 and s["cancelled"] == 1 and s["p50_s"] == 10.0


@pytest.mark.gpu
def test_cancel_mid_solve_and_waiting():
    """One request cancelled at its first Cd reading, another before it ever
    runs: both are reported cancelled (the first with the steps it made), the
    others end exactly as in a run without cancellations, and the log holds
    one JSON line per request."""
    from aeros_gb300 import serve
    reqs = _reqs(serve, 4)
    kw = dict(check_every=200, max_steps=600, chunk=100, tol=1e-3)
    base = {r.rid: r for r in serve.Server(**kw).run(reqs, realtime=False)["results"]}
    log = io.StringIO()
    srv = serve.Server(slots=3, log=log, **kw)
    victim, waiting = reqs[1].rid, reqs[3].rid
    srv.cancel(waiting)

    def check(rid, steps, cd):
        if rid == victim:
            srv.cancel(rid)

    out = srv.run(reqs, realtime=False, on_check=check)
    res = {r.rid: r for r in out["results"]}
    assert res[victim].cancelled and res[victim].steps == 200 and len(res[victim].cd_trace) == 1
    assert res[waiting].cancelled and res[waiting].steps == 0
    for rid in (reqs[0].rid, reqs[2].rid):
        assert not res[rid].cancelled
        assert (res[rid].steps, res[rid].cd) == (base[rid].steps, base[rid].cd)
        assert [c for _, c in res[rid].cd_trace][-1] == base[rid].cd
    lines = [json.loads(x) for x in log.getvalue().splitlines()]
    assert sorted(d["rid"] for d in lines) == sorted(r.rid for r in reqs)
    st = {d["rid"]: d["status"] for d in lines}
    assert st[victim] == "cancelled" and st[waiting] == "cancelled"
    assert all(d["mlups"] > 0 for d in lines if d["status"] != "cancelled")
    assert out["summary"]["requests"] == 2 and out["summary"]["cancelled"] == 2
