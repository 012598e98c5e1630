"""CUDA kernels against the reference's golden vectors (bit-exact) and against the oracle on
fresh seeded inputs: GPU encode + sidecar, query preparation (FHT, MT19937-64 dither, INT8
codes), the INT8 x MSB gate, the INT8 x remaining-3-bit traversal, the FP32 restore and the
residual4 rerank interval."""
import numpy as np
import pytest

from cases import kernel_inputs
from conftest import load_golden

pytestmark = pytest.mark.gpu

KERNEL_CASES = ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536"]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _space(torch, dim, center):
    from quantization_graph_gb300.space import RabitqSpace

    return RabitqSpace(dim, center)


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_encode_and_sidecar_bit_exact(cuda, name):
    torch = cuda
    g = load_golden(name)
    X, _ = kernel_inputs(int(g["dim"]), int(g["n"]), int(g["nq"]), int(g["seed"]))
    sp = _space(torch, int(g["dim"]), g["center"])
    compact, residual = sp.encode(torch.from_numpy(X).cuda())
    np.testing.assert_array_equal(compact.cpu().numpy(), g["compact"])
    np.testing.assert_array_equal(residual.cpu().numpy(), g["residual"])
    msb, factors = sp.export_paper_sidecar(torch.from_numpy(g["compact"]).cuda())
    np.testing.assert_array_equal(msb.cpu().numpy(), g["msb"])
    np.testing.assert_array_equal(factors.cpu().numpy(), g["factors"])


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_prepare_gate_distance_residual_bit_exact(cuda, name):
    torch = cuda
    g = load_golden(name)
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    sp = _space(torch, dim, g["center"])
    p = sp.prepare(torch.from_numpy(Q).cuda())
    np.testing.assert_array_equal(bits(p["rotated_residual"].cpu().numpy()), bits(g["rotated_residual"]))
    np.testing.assert_array_equal(p["codes"].cpu().numpy(), g["codes"])
    np.testing.assert_array_equal(bits(p["scalars"].cpu().numpy()), bits(g["scalars"]))
    np.testing.assert_array_equal(p["code_sum"].cpu().numpy(), g["code_sum"])
    qidx = np.repeat(np.arange(nq), n).astype(np.int32)
    ids = np.tile(np.arange(n), nq).astype(np.int32)
    msb = torch.from_numpy(g["msb"]).cuda()
    fac = torch.from_numpy(g["factors"]).cuda()
    comp = torch.from_numpy(g["compact"]).cuda()
    res = torch.from_numpy(g["residual"]).cuda()
    gate = sp.gate_pairs(p, qidx, ids, msb, fac, 1.9).cpu().numpy()
    np.testing.assert_array_equal(gate[:, :21], g["gate"].reshape(nq * n, -1)[:, :21])
    sip = gate[:, 4:8].copy().view(np.float32).ravel()
    d2 = sp.distance_pairs(p, qidx, ids, np.full(nq * n, 2, np.uint8), comp, sip).cpu().numpy()
    np.testing.assert_array_equal(bits(d2), bits(g["dist_mode2"].ravel()))
    d0 = sp.distance_pairs(p, qidx, ids, np.zeros(nq * n, np.uint8), comp, np.zeros(nq * n, np.float32))
    np.testing.assert_array_equal(bits(d0.cpu().numpy()), bits(g["dist_mode0"].ravel()))
    iv = sp.residual_pairs(p, qidx, ids, res, d0).cpu().numpy()
    np.testing.assert_array_equal(bits(iv), bits(g["residual_iv"].reshape(nq * n, 3)))


@pytest.mark.parametrize("dim", [64, 300, 960, 1024, 1536])
def test_encode_and_prepare_match_oracle_random(cuda, oracle, dim):
    torch = cuda
    rng = np.random.default_rng(dim)
    X = (rng.standard_normal((512, dim)) * rng.uniform(0.05, 3.0, dim)).astype(np.float32)
    X[7] = 0.0  # zero row: residual equals minus the centre
    c = X.mean(0).astype(np.float32)
    X[9] = c     # a row equal to the centre: zero residual norm
    o = oracle.Oracle(dim, c)
    sp = _space(torch, dim, c)
    compact, residual = sp.encode(torch.from_numpy(X).cuda())
    oc, orr = o.encode(X)
    np.testing.assert_array_equal(compact.cpu().numpy(), oc)
    np.testing.assert_array_equal(residual.cpu().numpy(), orr)
    Q = (rng.standard_normal((64, dim)) * 2).astype(np.float32)
    Q[3] = c  # query at the centre: zero residual, zero scale
    p = sp.prepare(torch.from_numpy(Q).cuda())
    for i in range(len(Q)):
        po = o.prepare(Q[i])
        np.testing.assert_array_equal(p["codes"][i].cpu().numpy(), po["codes"])
        assert int(p["code_sum"][i]) == po["code_sum"]
        sc = p["scalars"][i].cpu().numpy()
        np.testing.assert_array_equal(bits(sc), bits(np.array([po["query_norm_sqr"], po["query_norm"],
                                                               po["half_sum"], po["scale"]], np.float32)))


def test_center_mean_matches_sequential_f32(cuda):
    torch = cuda
    from quantization_graph_gb300.space import train_global_center

    rng = np.random.default_rng(3)
    X = rng.standard_normal((5000, 96)).astype(np.float32)
    got = train_global_center(torch.from_numpy(X).cuda()).cpu().numpy()
    acc = np.zeros(96, np.float32)
    for row in X:
        acc = (acc + row).astype(np.float32)
    want = (acc * (np.float32(1.0) / np.float32(5000))).astype(np.float32)
    np.testing.assert_array_equal(bits(got), bits(want))
