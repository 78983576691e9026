"""Batched plans (one persistent launch over many uneven requests, graph
replay, autotuned launch shapes) against the chain of reference calls each
request stands for, computed by the oracle."""
import numpy as np
import pytest

import oracle
import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import batch

pytestmark = pytest.mark.gpu
U = np.uint64


def dev(a):
    import torch
    if a is None:
        return None
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int64) if a.dtype == np.uint64 else a).cuda()


def net_chain(req):
    """The reference chain for one digital-net request, on the oracle."""
    r, n, d, alpha, mmax = req["r"], req["n"], req["d"], req["alpha"], req["mmax"]
    d_pre = d * alpha
    C = req["C"]
    r_C = req["r_C"]
    bits = req["tmax"]
    if req.get("S") is not None:
        Cl = np.empty((r, d_pre, mmax), U)
        oracle.call("dnb2_linear_matrix_scramble", U(r), U(d_pre), U(mmax), U(r_C), U(req["tmax_new"]), req["S"],
                    C, Cl)
        C, r_C, bits = Cl, r, req["tmax_new"]
    if alpha > 1:
        Ca = np.empty((r_C, d, mmax), U)
        oracle.call("dnb2_interlace", U(r_C), U(d), U(mmax), U(d_pre), U(bits), U(req["tmax_alpha"]), U(alpha),
                    C, Ca)
        C = Ca
    # generation with r randomisations (matrix set l % r_C)
    Cr = np.stack([C[l % r_C] for l in range(r)])
    xb = np.empty((r, n, d), U)
    oracle.call("dnb2_gen_gray" if req["order"] == "gray" else "dnb2_gen_natural", U(r), U(n), U(d),
                U(req["n_start"]), U(mmax), Cr, xb)
    if req.get("shifts") is not None:
        xr = np.empty((r, n, d), U)
        oracle.call("dnb2_digital_shift", U(r), U(n), U(d), U(r), req["lshifts"], xb, req["shifts"], xr)
        xb = xr
    xf = None
    if req.get("tmaxes") is not None:
        xf = np.empty((r, n, d))
        oracle.call("dnb2_integer_to_float", U(r), U(n), U(d), req["tmaxes"], xb, xf)
    return xb, xf


def make_net_requests(rng, count):
    reqs = []
    for k in range(count):
        alpha = [1, 2, 3][k % 3]
        d = int(rng.choice([1, 3, 8, 16, 33, 64, 70]))
        m = int(rng.integers(4, 14))
        n_start = 0 if k % 4 else (1 << (m - 2))
        n = (1 << m) - n_start if k % 5 else int(rng.integers(1, 1 << m))
        order = "gray" if (k % 2 or k % 5 == 0) else "natural"
        if order == "natural" and n_start + n != (1 << m):
            n = (1 << m) - n_start
        mmax = m + 1
        tmax = 32 if k % 2 else 63
        r, r_C = int(rng.integers(1, 4)), 1
        req = dict(r=r, n=n, d=d, alpha=alpha, mmax=mmax, n_start=n_start, order=order, r_C=r_C, tmax=tmax,
                   tmax_new=64, tmax_alpha=min(alpha * 64, 64))
        req["C"] = q.random_tbit_uint64s(rng, tmax, (r_C, d * alpha, mmax))
        if k % 3 != 2:
            req["S"] = q.dnb2_get_linear_scramble_matrix(rng, r, d * alpha, tmax, 64, False)
        else:
            req["tmax_alpha"] = min(alpha * tmax, 64)
        if k % 4 != 3:
            req["shifts"] = q.dnb2_get_digital_shifts(rng, r, d, 64)
            req["lshifts"] = np.array([0, 1, 5][:r], U)
        if k % 2 == 0:
            req["tmaxes"] = np.full(r, 64, U)
        reqs.append(req)
    return reqs


def to_plan_requests(reqs):
    import torch
    out = []
    for req in reqs:
        r, n, d = req["r"], req["n"], req["d"]
        p = dict(req)
        for key in ("C", "S", "shifts", "lshifts", "tmaxes"):
            p[key] = dev(req.get(key))
        p["xb"] = torch.full((r * n * d,), -1, dtype=torch.int64, device="cuda")
        p["x"] = torch.full((r * n * d,), -1.0, dtype=torch.float64, device="cuda") if req.get("tmaxes") is not None \
            else None
        out.append(p)
    return out


def check_net(plan_reqs, reqs):
    for p, req in zip(plan_reqs, reqs):
        xb, xf = net_chain(req)
        got = p["xb"].cpu().numpy().view(U).reshape(xb.shape)
        assert np.array_equal(got, xb)
        if xf is not None:
            gotf = p["x"].cpu().numpy().reshape(xf.shape)
            assert np.array_equal(gotf.view(U), xf.view(U))


def test_net_plan_uneven_requests_run_and_replay():
    import torch
    rng = np.random.Generator(np.random.SFC64(31))
    reqs = make_net_requests(rng, 12)
    preqs = to_plan_requests(reqs)
    plan = batch.NetPlan(preqs)
    info = plan.info()
    assert info["launches"] == 2 and info["tiles"] > 0
    plan.run()
    torch.cuda.synchronize()
    check_net(preqs, reqs)
    # relaunch with outputs cleared: the work queue must have reset itself
    for p in preqs:
        p["xb"].fill_(-1)
    plan.run()
    plan.run()
    torch.cuda.synchronize()
    check_net(preqs, reqs)
    s = torch.cuda.Stream()
    for _ in range(3):
        for p in preqs:
            p["xb"].fill_(-1)
        torch.cuda.synchronize()
        plan.graph_launch(s)
        s.synchronize()
        check_net(preqs, reqs)


def test_net_plan_tuning_shapes_stay_exact():
    import torch
    rng = np.random.Generator(np.random.SFC64(32))
    reqs = make_net_requests(rng, 6)
    preqs = to_plan_requests(reqs)
    plan = batch.NetPlan(preqs)
    for ctas, chunk, tile in [(1, 1, 1 << 10), (8, 16, 1 << 20), (2, 3, 5000)]:
        for p in preqs:
            p["xb"].fill_(-1)
        plan.set_tuning(ctas, chunk, tile)
        plan.run()
        torch.cuda.synchronize()
        check_net(preqs, reqs)


def test_autotune_and_cache(tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("QMCGB_TUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.Generator(np.random.SFC64(33))
    reqs = make_net_requests(rng, 4)
    preqs = to_plan_requests(reqs)
    plan = batch.NetPlan(preqs)
    best = plan.tune(reps=1)
    assert len(best) == 4 and best[3] > 0
    assert (tmp_path / "tune.json").exists()
    again = batch.NetPlan(preqs).tune(reps=1)  # same shape class: from the cache
    assert list(again) == list(best)
    for p in preqs:
        p["xb"].fill_(-1)
    plan.run()
    torch.cuda.synchronize()
    check_net(preqs, reqs)


def lat_chain(req):
    r, n, d = req["r"], req["n"], req["d"]
    x = np.empty((r, n, d))
    oracle.call("lat_gen_gray" if req["order"] == "gray" else "lat_gen_natural", U(r), U(n), U(d),
                U(req["n_start"]), req["g"], x)
    if req.get("shifts") is None:
        return x
    xr = np.empty((r, n, d))
    oracle.call("lat_shift_mod_1", U(r), U(n), U(d), U(r), x, req["shifts"], xr)
    return xr


def test_lat_plan_uneven_requests():
    import torch
    rng = np.random.Generator(np.random.SFC64(34))
    reqs, preqs = [], []
    for k in range(10):
        m = int(rng.integers(3, 15))
        d = int(rng.choice([1, 2, 5, 64, 100]))
        order = "gray" if k % 3 else "natural"
        n_start = 0 if order == "natural" or k % 2 else int(rng.integers(0, 1000))
        n = 1 << m
        r = int(rng.integers(1, 4))
        g = (rng.integers(0, 1 << 19, (r, d)) * 2 + 1).astype(U)
        if k == 4:
            g[0, 0] = U((1 << 45) + 1)  # FP64 column
        req = dict(r=r, n=n, d=d, n_start=n_start, order=order, g=g)
        if k % 4:
            req["shifts"] = q.lat_get_shifts(rng, r, d)
        reqs.append(req)
        p = dict(req, g=dev(g), shifts=dev(req.get("shifts")),
                 x=torch.full((r * n * d,), -1.0, dtype=torch.float64, device="cuda"))
        preqs.append(p)
    plan = batch.LatPlan(preqs)
    s = torch.cuda.Stream()
    for mode in ("run", "graph", "graph"):
        for p in preqs:
            p["x"].fill_(-1.0)
        torch.cuda.synchronize()
        if mode == "run":
            plan.run(s)
        else:
            plan.graph_launch(s)
        s.synchronize()
        for p, req in zip(preqs, reqs):
            want = lat_chain(req)
            got = p["x"].cpu().numpy().reshape(want.shape)
            assert np.array_equal(got.view(U), want.view(U))
