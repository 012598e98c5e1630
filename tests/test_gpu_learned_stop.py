"""Learned early termination: the network's forward, backward and Adam kernels against an FP64
numpy restatement, trace collection, and what the trained stop gains over plain fixed-L search
on a reference-built graph."""
import numpy as np
import pytest

from cases import SEARCH_CASES
from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_mlp_forward_backward_adam_match_fp64(cuda):
    torch = cuda
    import mlp_ref
    from quantization_graph_gb300 import learned_stop as ls

    rng = np.random.default_rng(0)
    x = rng.standard_normal((257, 8)).astype(np.float32) * 3 + 1
    y = (rng.random(257) < 0.4).astype(np.float32)
    y_budget = (np.log(rng.integers(8, 900, 257)) + 0.0).astype(np.float32)
    norm = np.concatenate([x.mean(0), 1 / x.std(0)]).astype(np.float32)
    master = ls.init_weights(3)
    w = ls.to_bf16_bits(master)
    wb = mlp_ref.bf16_round(master.cpu().numpy())
    np.testing.assert_array_equal(w.cpu().numpy().view(np.uint16).astype(np.uint32) << 16,
                                  wb.astype(np.float32).view(np.uint32))
    tn = torch.from_numpy(norm).cuda()
    z = ls.forward(w, tn, torch.from_numpy(x)).cpu().numpy()
    z_ref, _ = mlp_ref.forward(wb, norm.astype(np.float64), x)
    np.testing.assert_allclose(z, z_ref, rtol=1e-4, atol=1e-4)
    loss, grad = ls.loss_and_grad(w, tn, torch.from_numpy(x), torch.from_numpy(y))
    l_ref, g_ref = mlp_ref.loss_and_grad(wb, norm.astype(np.float64), x, y)
    assert abs(float(loss) - l_ref) < 1e-4 * max(1.0, abs(l_ref))
    g = grad.cpu().numpy()
    scale = np.abs(g_ref).max()
    np.testing.assert_allclose(g, g_ref, rtol=1e-3, atol=1e-5 * scale)
    # the hop budget's squared-error loss and gradient
    lm, gm = ls.loss_and_grad(w, tn, torch.from_numpy(x), torch.from_numpy(y_budget), kind=ls.KIND_BUDGET)
    lm_ref, gm_ref = mlp_ref.loss_and_grad(wb, norm.astype(np.float64), x, y_budget, mse=True)
    assert abs(float(lm) - lm_ref) < 1e-4 * max(1.0, abs(lm_ref))
    np.testing.assert_allclose(gm.cpu().numpy(), gm_ref, rtol=1e-3, atol=1e-5 * np.abs(gm_ref).max())
    # one Adam step
    from quantization_graph_gb300 import _native as N
    import ctypes as C

    lib = N.load()
    m = torch.zeros_like(master)
    v = torch.zeros_like(master)
    m0 = master.cpu().numpy().astype(np.float64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.qg_mlp_adam(C.c_void_p(master.data_ptr()), C.c_void_p(w.data_ptr()), C.c_void_p(grad.data_ptr()),
                           C.c_void_p(m.data_ptr()), C.c_void_p(v.data_ptr()), 1e-2, 0.9, 0.999, 1e-8, 1,
                           stream) == 0
    want, _, _ = mlp_ref.adam(m0, g.astype(np.float64), 0, 0, 1e-2, 0.9, 0.999, 1e-8, 1)
    np.testing.assert_allclose(master.cpu().numpy(), want, rtol=1e-5, atol=1e-6)


def _index(torch):
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden("search_c1")
    sp = RabitqSpace(128, g["center"])
    return g, OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])


def test_learned_stop_saves_hops_at_equal_recall(cuda, oracle):
    torch = cuda
    from quantization_graph_gb300 import learned_stop as ls
    from quantization_graph_gb300 import synthetic

    g, ix = _index(torch)
    X, _ = SEARCH_CASES["search_c1"]()
    _, cent = synthetic.gmm(1, 128, components=64, sigma=0.3, seed=11)
    train_q, _ = synthetic.gmm(3000, 128, sigma=0.3, seed=101, centres=cent)
    test_q, _ = synthetic.gmm(1000, 128, sigma=0.3, seed=102, centres=cent)
    L = 80
    tq = torch.from_numpy(train_q).cuda()
    truth = ix.search(tq, k=10, l_value=L, with_stats=False).ids.to(torch.int32)
    tr = ls.collect_traces(ix, tq, truth, k=10, l_value=L, every=2)
    labels = tr.classifier_labels()
    assert tr.features.shape[0] == labels.shape[0] > 10_000
    assert 0.05 < float(labels.mean()) < 0.95
    model = ls.train(tr.features, labels, epochs=6, batch=4096, every=2, min_hops=4)
    o = oracle.Oracle(128, g["center"])
    gt, _ = o.exact_knn(X, test_q, 10)
    qq = torch.from_numpy(test_q).cuda()
    plain = ix.search(qq, k=10, l_value=L)
    rec_plain = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(plain.ids.cpu().numpy(), gt)])
    hops_plain = plain.stats["hops"].mean()
    stats = torch.empty((len(test_q), 9), dtype=torch.int64, device="cuda")
    best = None
    for thr in (0.5, 0.7, 0.8, 0.9, 0.95, 0.98):
        ids, _ = ls.search(ix, qq, model, thr, k=10, l_value=L, stats_out=stats)
        rec = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(ids.cpu().numpy(), gt)])
        hops = stats[:, 2].double().mean().item()
        if rec >= rec_plain - 0.002 and (best is None or hops < best[1]):
            best = (thr, hops, rec)
    assert best is not None, "no threshold kept recall within 0.002 of fixed-L"
    assert best[1] <= 0.9 * hops_plain, (best, hops_plain, rec_plain)


def test_in_kernel_stop_matches_standalone_forward(cuda):
    """The search kernel's stop decision (network staged in shared memory) equals the standalone
    forward kernel applied to the trace of the same search: each query stops at the first
    checkpoint whose logit exceeds the threshold, else runs to the end."""
    torch = cuda
    from quantization_graph_gb300 import learned_stop as ls
    from quantization_graph_gb300 import synthetic

    g, ix = _index(torch)
    _, cent = synthetic.gmm(1, 128, components=64, sigma=0.3, seed=11)
    train_q, _ = synthetic.gmm(1500, 128, sigma=0.3, seed=201, centres=cent)
    test_q, _ = synthetic.gmm(400, 128, sigma=0.3, seed=202, centres=cent)
    L, every, min_hops, thr = 80, 2, 4, 0.8
    tq = torch.from_numpy(train_q).cuda()
    truth = ix.search(tq, k=10, l_value=L, with_stats=False).ids.to(torch.int32)
    tr = ls.collect_traces(ix, tq, truth, k=10, l_value=L, every=every)
    model = ls.train(tr.features, tr.classifier_labels(), epochs=2, batch=4096, every=every, min_hops=min_hops)
    qq = torch.from_numpy(test_q).cuda()
    truth_te = ix.search(qq, k=10, l_value=L, with_stats=False).ids.to(torch.int32)
    # per-checkpoint rows of the plain search, query by query
    import ctypes as C

    from quantization_graph_gb300 import _native as N
    from quantization_graph_gb300.space import _ptr, _stream

    nq, cap = len(test_q), (4 * L) // every + 8
    feat = torch.empty((nq, cap, 8), dtype=torch.float32, device="cuda")
    lab = torch.empty((nq, cap), dtype=torch.float32, device="cuda")
    cnt = torch.empty(nq, dtype=torch.int32, device="cuda")
    ids = torch.empty((nq, 10), dtype=torch.int32, device="cuda")
    dists = torch.empty((nq, 10), dtype=torch.float32, device="cuda")
    stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda")
    params = N.SearchParams(10, L, 1, 1.9, 100, 0, 0)
    treq = N.TraceRequest(truth_te.data_ptr(), 10, every, cap, feat.data_ptr(), lab.data_ptr(), cnt.data_ptr())
    lib = N.load()
    N.check(lib.qg_search_batch_learned(ix.handle, _ptr(qq), nq, C.byref(params), None, None, 10, _ptr(ids),
                                        _ptr(dists), _ptr(stats), None, C.byref(treq), _stream()), "trace")
    full_hops = stats[:, 2].cpu().numpy()
    logits = ls.forward(model.weights, model.norm, feat.reshape(-1, 8)).reshape(nq, cap).cpu().numpy()
    cnt = cnt.cpu().numpy()
    z_thr = np.log(np.float32(thr) / (np.float32(1.0) - np.float32(thr)))
    want = full_hops.copy()
    for q in range(nq):
        for r in range(cnt[q]):
            h = (r + 1) * every
            if h >= min_hops and logits[q, r] > z_thr:
                want[q] = h
                break
    stats2 = torch.empty((nq, 9), dtype=torch.int64, device="cuda")
    ls.search(ix, qq, model, thr, k=10, l_value=L, stats_out=stats2)
    got = stats2[:, 2].cpu().numpy()
    assert (want < full_hops).sum() > 20, "the threshold should stop some queries early"
    np.testing.assert_array_equal(got, want)


def test_in_kernel_budget_matches_standalone_forward(cuda):
    """The hop budget in the search kernel: each query stops at the first hop h >= scale *
    exp(output), the output re-predicted at every checkpoint (or taken at the first one only),
    exactly as the standalone forward kernel over the plain search's trace says; the trace's
    targets (log of the first hop whose rerank window holds the whole result) are consistent."""
    torch = cuda
    import ctypes as C

    from quantization_graph_gb300 import _native as N
    from quantization_graph_gb300 import learned_stop as ls
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.space import _ptr, _stream

    g, ix = _index(torch)
    _, cent = synthetic.gmm(1, 128, components=64, sigma=0.3, seed=11)
    train_q, _ = synthetic.gmm(1500, 128, sigma=0.3, seed=301, centres=cent)
    test_q, _ = synthetic.gmm(400, 128, sigma=0.3, seed=302, centres=cent)
    L, every, min_hops, scale = 80, 2, 4, 0.9
    tq = torch.from_numpy(train_q).cuda()
    truth = ix.search(tq, k=10, l_value=L, with_stats=False).ids.to(torch.int32)
    tr = ls.collect_traces(ix, tq, truth, k=10, l_value=L, every=every)
    y = tr.budget_targets()
    h = tr.hops_needed()
    assert bool((h <= tr.final_hops).all()) and bool((h >= 1).all())
    assert float((h < tr.final_hops).float().mean()) > 0.5  # most queries hold their result before the end
    qq = torch.from_numpy(test_q).cuda()
    truth_te = ix.search(qq, k=10, l_value=L, with_stats=False).ids.to(torch.int32)
    te = ls.collect_traces(ix, qq, truth_te, k=10, l_value=L, every=every, cap=(4 * L) // every + 8)
    nq = len(test_q)
    for once in (False, True):
        model = ls.train(tr.features, y, epochs=2, batch=4096, every=every, min_hops=min_hops,
                         kind=ls.KIND_BUDGET, predict_once=once)
        z = ls.forward(model.weights, model.norm, te.features).cpu().numpy()
        full = te.final_hops.cpu().numpy()
        rows_q = te.query.cpu().numpy()
        rows_h = te.hop.cpu().numpy()
        zq = {}
        for r in range(len(z)):
            zq[(rows_q[r], rows_h[r])] = z[r]
        # replay the kernel's rule hop by hop: at a checkpoint (hop % every == 0, hop >= min_hops)
        # the budget is (re)predicted, then the query stops at the first hop >= the budget
        want = full.copy()
        clear = np.ones(nq, bool)  # budgets within float rounding of the deciding hop are skipped
        for q in range(nq):
            budget = 0.0
            for hop in range(1, int(full[q]) + 1):
                if hop % every == 0 and hop >= min_hops and (q, hop) in zq and not (once and budget > 0):
                    budget = float(np.float32(np.exp(np.float32(min(zq[(q, hop)], 30.0)))) * np.float32(scale))
                if budget > 0 and abs(hop - budget) < 1e-3 * budget:
                    clear[q] = False
                if budget > 0 and hop >= budget:
                    want[q] = hop
                    break
        stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda")
        ls.search(ix, qq, model, scale, k=10, l_value=L, stats_out=stats)
        got = stats[:, 2].cpu().numpy()
        assert clear.sum() > 0.9 * nq
        want, got, full = want[clear], got[clear], full[clear]
        assert (want < full).sum() > 20, "the budget should stop some queries early"
        np.testing.assert_array_equal(got, want)
