"""GPU: continuous-batching serving loop.  Every request's result in the mix
equals the same request run alone: sampling bit-exactly (same seed, the
packed launch runs the per-sample code of the single launch), CP-ALS up to
the order of floating-point atomic additions in the MTTKRP (factors within
1e-9 of the largest entry, fit within 1e-9).  The HBM budget is never
exceeded and concurrent sampling requests share packed launches."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ftl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fast_tensor_leverage_gb300 as m
    return m


def _sparse(rng, dims, nnz):
    flat = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    return idx, np.log1p(rng.lognormal(0.0, 1.0, size=nnz))


def _requests(S):
    rng = np.random.default_rng(12)
    reqs = []
    specs = [(3, 2000, 16, 3000, 4, "fp32"), (4, 900, 16, 5000, 1, "fp32"), (3, 40000, 32, 8000, 9, "fp32"),
             (5, 300, 8, 2000, 0, "fp64"), (3, 7000, 16, 1000, 2, "fp32"), (6, 120, 8, 4000, 9, "fp32")]
    for n, (N, I, R, J, j, prec) in enumerate(specs):
        factors = [rng.normal(size=(I + 37 * k, R)) for k in range(N)]
        reqs.append(S.SampleRequest(factors, J, j, prec, seed=100 + n))
    for n, (dims, nnz, R, J) in enumerate([([40, 30, 20], 2000, 8, 400), ([25, 60, 35], 3000, 6, 300)]):
        idx, vals = _sparse(rng, dims, nnz)
        reqs.append(S.ALSRequest(idx, vals, dims, R, J, sweeps=3, precision="fp64", seed=5 + n,
                                 sampler_seed=9 + n))
    return reqs


def test_mix_equals_alone(ftl):
    from fast_tensor_leverage_gb300 import serving as S
    reqs = _requests(S)
    sizes = [S.estimate_bytes(r) for r in reqs]
    budget = sum(sorted(sizes)[-3:])  # forces some requests to wait
    eng = S.ServingEngine(budget, max_active=8)
    # a burst of three requests (two share R = 16 and pack into one launch),
    # then the rest spread out while those are on the device
    arrivals = [(0.0 if i < 3 else 0.002 * i, r) for i, r in enumerate(reqs)]
    done = eng.run(arrivals)
    assert len(done) == len(reqs)
    assert eng.max_in_use <= budget
    by_id = {h.rid: h for h in done}
    for rid, r in enumerate(reqs):
        res = by_id[rid].result
        if isinstance(r, S.SampleRequest):
            s = ftl.Sampler(r.factors, r.J, r.factors[0].shape[1], "efficient", precision=r.precision, seed=r.seed)
            samples, h, w = s.draw(r.j)
            N = len(r.factors)
            rows = [k for k in range(N) if k != r.j]
            assert np.array_equal(res["samples"][rows], samples.cpu().numpy().view(np.uint64)[rows])
            assert np.array_equal(res["h"], h.cpu().numpy())
            assert np.array_equal(res["weights"], w.cpu().numpy())
        else:
            U = S.GaussianFactors(r.dims, r.R, seed=r.seed).materialize(torch.device("cuda", 0))
            lr = ftl.LowRankTensor(r.R, U, sync_host=False)
            lr.renormalize_columns(-1)
            sp = ftl.SparseTensor(r.idx, r.vals, "sort", dims=r.dims)
            als = ftl.ALS(lr, sp)
            als.initialize_ds_als(r.J, "efficient", precision=r.precision, seed=r.sampler_seed)
            for _ in range(r.sweeps):
                for j in range(len(r.dims)):
                    als.execute_ds_als_update(j, True, True)
            for k in range(len(r.dims)):
                ref = lr.U_dev[k].cpu().numpy()
                np.testing.assert_allclose(res["U"][k], ref, rtol=0, atol=1e-9 * np.abs(ref).max())
            resid = sp.compute_residual_normsq(lr.sigma_dev, lr.U_dev)
            fit = 1.0 - np.sqrt(max(resid, 0.0) / sp.get_normsq())
            assert abs(res["fit"] - fit) <= 1e-9
    assert eng.packed_launches < sum(isinstance(r, S.SampleRequest) for r in reqs)
    lat = S.latency_stats(done)
    assert lat["count"] == len(reqs) and lat["p99_ms"] >= lat["p50_ms"] > 0


def test_captured_als_sweep_equals_eager(ftl):
    rng = np.random.default_rng(4)
    dims, R, J = [30, 45, 25], 7, 350
    flat = rng.choice(int(np.prod(dims)), size=2500, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    vals = rng.random(2500) + 0.5
    out = []
    for graph in (False, True):
        r2 = np.random.default_rng(8)
        U = [r2.normal(size=(d, R)) for d in dims]
        lr = ftl.LowRankTensor(R, U, sync_host=False)
        lr.renormalize_columns(-1)
        sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
        als = ftl.ALS(lr, sp)
        als.initialize_ds_als(J, "efficient", precision="fp64", seed=21)
        for j in range(3):
            als.execute_ds_als_update(j, True, True)
        if graph:
            als.capture_sweep()
            for _ in range(3):
                als.replay_sweep()
        else:
            for _ in range(3):
                for j in range(3):
                    als.execute_ds_als_update(j, True, True)
        torch.cuda.synchronize()
        out.append([u.cpu().numpy() for u in lr.U_dev])
    for a, b in zip(*out):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-9 * np.abs(b).max())


def _packed(ftl, samplers, js, cancel=None, budget_ns=0, ctl=True):
    """One packed draw of the samplers through the C ABI (with or without
    the serving controls); returns the statuses (or None)."""
    import ctypes
    from fast_tensor_leverage_gb300 import _lib
    n = len(samplers)
    plans = (ctypes.POINTER(_lib.KRPPlan) * n)(*[ctypes.pointer(s._plan) for s in samplers])
    jj = (ctypes.c_uint32 * n)(*js)
    smp = (ctypes.c_void_p * n)(*[s.samples_dev.data_ptr() for s in samplers])
    hh = (ctypes.c_void_p * n)(*[s.h_dev.data_ptr() for s in samplers])
    ww = (ctypes.c_void_p * n)(*[s.weights_dev.data_ptr() for s in samplers])
    seeds = (ctypes.c_uint64 * n)(*[s.seed for s in samplers])
    ctrs = (ctypes.c_uint64 * n)(*[0] * n)
    st = torch.cuda.current_stream().cuda_stream
    for s, j in zip(samplers, js):
        _lib.call("ftl_krp_compute_m", ctypes.byref(s._plan), j, st)
    if not ctl:
        _lib.call("ftl_krp_sample_packed", plans, n, jj, smp, hh, ww, None, seeds, ctrs, st)
        torch.cuda.synchronize()
        return None
    status = torch.zeros(72, dtype=torch.uint8, device="cuda")
    flags = (ctypes.c_void_p * n)(*[(c.data_ptr() if c is not None else None) for c in (cancel or [None] * n)])
    _lib.call("ftl_krp_sample_packed_ctl", plans, n, jj, smp, hh, ww, None, seeds, ctrs, flags, budget_ns,
              status.data_ptr(), st)
    torch.cuda.synchronize()
    return status.cpu().numpy()[8:].view(np.uint32)[:n].tolist()


def test_packed_draw_controls_cancel_and_timeout(ftl):
    """Serving controls of the packed draw, without a GPU fault or wait:
    a request whose host flag is set before the launch is skipped with
    FTL_E_CANCELLED and leaves its outputs untouched while the other request
    is bit-identical to the uncontrolled launch; a 1 ns budget stops every
    request of a large launch with FTL_E_TIMEOUT; a generous budget changes
    nothing."""
    from fast_tensor_leverage_gb300 import _lib
    rng = np.random.default_rng(44)
    for R, prec in ((32, "fp32"), (16, "fp32"), (8, "fp64")):
        U1 = [rng.normal(size=(3000, R)) for _ in range(3)]
        U2 = [rng.normal(size=(2000, R)) for _ in range(3)]
        a = ftl.Sampler(U1, 20000, R, "efficient", precision=prec, seed=1, overlap_computem=False)
        b = ftl.Sampler(U2, 30000, R, "efficient", precision=prec, seed=2, overlap_computem=False)
        _packed(ftl, [a, b], [4, 4], ctl=False)
        ref_a = (a.samples_dev.clone(), a.h_dev.clone(), a.weights_dev.clone())
        # cancelled before the launch
        b.samples_dev.fill_(-7)
        flag = torch.ones(1, dtype=torch.int32, pin_memory=True)
        a.samples_dev.zero_()
        st = _packed(ftl, [a, b], [4, 4], cancel=[None, flag])
        assert st == [0, _lib.FTL_E_CANCELLED], (R, st)
        assert torch.equal(a.samples_dev, ref_a[0]) and torch.equal(a.h_dev, ref_a[1])
        assert torch.equal(a.weights_dev, ref_a[2])
        assert bool((b.samples_dev == -7).all())
        # a generous budget: nothing stops, results as without controls
        st = _packed(ftl, [a, b], [4, 4], budget_ns=10**12)
        assert st == [0, 0] and torch.equal(a.samples_dev, ref_a[0])
        # 1 ns: every request times out
        big = ftl.Sampler([rng.normal(size=(5000, R)) for _ in range(3)], 200000, R, "efficient", precision=prec,
                          seed=3, overlap_computem=False)
        st = _packed(ftl, [big, a], [4, 4], budget_ns=1)
        assert st == [_lib.FTL_E_TIMEOUT, _lib.FTL_E_TIMEOUT], (R, st)


def test_engine_cancel(ftl):
    """ServingEngine.cancel: a request cancelled while pending finishes
    with status "cancelled" and no device work; the others complete with
    their results."""
    from fast_tensor_leverage_gb300 import serving as S
    rng = np.random.default_rng(3)
    eng = S.ServingEngine(8 << 30, max_active=4)
    hs = [eng.submit(S.SampleRequest([rng.normal(size=(1000, 8)) for _ in range(3)], 2000, 4, "fp32", seed=k))
          for k in range(3)]
    hs[1].cancel()
    while not eng.idle():
        eng.tick()
    assert hs[1].status == "cancelled" and hs[1].result == {"status": "cancelled"}
    for k in (0, 2):
        assert hs[k].status == "ok" and hs[k].result["samples"].shape == (3, 2000)


def test_engine_request_budget_times_out(ftl):
    """A request whose device-time budget (1 ns) is shorter than its draw
    finishes with status "timeout" and no results."""
    from fast_tensor_leverage_gb300 import serving as S
    rng = np.random.default_rng(4)
    eng = S.ServingEngine(8 << 30, max_active=4)
    h = eng.submit(S.SampleRequest([rng.normal(size=(4000, 16)) for _ in range(3)], 300000, 9, "fp32", seed=1,
                                   budget_s=1e-9))
    while not eng.idle():
        eng.tick()
    assert h.status == "timeout" and h.result == {"status": "timeout"}
