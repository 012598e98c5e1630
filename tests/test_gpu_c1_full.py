"""The CPU-runnable workload at its stated size, end to end on the GPU against the oracle (the
reference's path restated, pinned to the reference's own bridge): 20,000 x 128 vectors from a
seeded 64-component Gaussian mixture (centres N(0,1), sigma 0.3), 500 queries from the same
mixture; GPU encode and sidecar, the reference's Vamana build on the GPU (M=32, L_build=100,
alpha 1.2, refine 1, prune cap 256, early stop 2, batch 4096), searches at k=10 and
L in {20, 40, 80} with the residual4 top-100 rerank. Records, graph, ids, distance bits and the
9 counters must all equal the oracle's; recall is measured against exact FP64 brute force."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_c1_at_full_size_equals_the_oracle(cuda, oracle):
    torch = cuda
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.graph_build import build_vamana
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace, train_global_center

    X, cent = synthetic.gmm(20000, 128, components=64, sigma=0.3, seed=11)
    Q, _ = synthetic.gmm(500, 128, sigma=0.3, seed=12, centres=cent)
    center = train_global_center(torch.from_numpy(X).cuda()).cpu().numpy()  # all rows: N <= 100k
    sp = RabitqSpace(128, center)
    o = oracle.Oracle(128, center)
    compact, residual = sp.encode(torch.from_numpy(X))
    oc, orr = o.encode(X)
    np.testing.assert_array_equal(compact.cpu().numpy(), oc)
    np.testing.assert_array_equal(residual.cpu().numpy(), orr)
    msb, factors = sp.export_paper_sidecar(compact)
    om, of = o.sidecar(oc)
    np.testing.assert_array_equal(msb.cpu().numpy(), om)
    np.testing.assert_array_equal(factors.cpu().numpy(), of)
    kw = dict(r=32, l_build=100, alpha=1.2, beam=1, batch=4096, refine=1, cap=256, stop_hops=2)
    deg, edges, _ = build_vamana(sp, compact, **kw)
    odeg, oedges, _ = o.build_graph(oc, **kw)
    deg = deg.cpu().numpy().view(np.uint32)
    edges = edges.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(deg, odeg)
    for i in range(len(deg)):
        np.testing.assert_array_equal(edges[i, :deg[i]], oedges[i, :odeg[i]])
    index = OursIndex(sp, compact, residual, msb, factors, deg, edges)
    oindex = dict(compact=oc, residual=orr, msb=om, factors=of, degrees=odeg, edges=oedges,
                  total_points=len(X), base_points=len(X))
    gt, _ = o.exact_knn(X, Q, 10)
    recalls = []
    for L in (20, 40, 80):
        r = index.search(torch.from_numpy(Q).cuda(), k=10, l_value=L)
        oi, od, ost = o.search(Q, oindex, k=10, L=L)
        ids = r.ids.cpu().numpy().astype(np.uint32)
        np.testing.assert_array_equal(ids, oi)
        np.testing.assert_array_equal(r.distances.cpu().numpy().view(np.uint32), od.view(np.uint32))
        for f in ost.dtype.names:
            np.testing.assert_array_equal(r.stats[f], ost[f], err_msg=f)
        recalls.append(float(np.mean([len(set(a) & set(b)) / 10 for a, b in zip(ids, gt)])))
    assert recalls[0] <= recalls[1] <= recalls[2] and recalls[2] > 0.9, recalls
    print(f"recall@10 at L = 20 / 40 / 80: {recalls}")
