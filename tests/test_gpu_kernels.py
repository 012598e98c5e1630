"""CUDA kernels against the reference's golden vectors (bit-exact) and against the oracle on
fresh seeded inputs: GPU encode + sidecar, query preparation (FHT, MT19937-64 dither, INT8
codes), the INT8 x MSB gate, the INT8 x remaining-3-bit traversal, the FP32 restore and the
residual4 rerank interval."""
import numpy as np
import pytest

from cases import kernel_inputs
from conftest import load_golden

pytestmark = pytest.mark.gpu

KERNEL_CASES = ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536", "kernels_d128_int4",
                "kernels_d1536_int4"]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _space(torch, dim, center, codec=3):
    from quantization_graph_gb300.space import RabitqSpace

    return RabitqSpace(dim, center, codec=codec)


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
    sp = _space(torch, dim, g["center"], int(g.get("codec", 3)))
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


def test_dither_decision_near_integer_boundaries(cuda):
    """The FP32 dither decision equals floor(double(x)/double(scale) + u) exactly, including
    draws placed on and within a few ulps of integer boundaries (where it must fall back)."""
    torch = cuda
    import ctypes as C

    from quantization_graph_gb300 import _native as N

    rng = np.random.default_rng(11)
    m = 20000
    scale = rng.uniform(0.001, 4.0, m).astype(np.float32)
    K = rng.integers(0, 2**64 - 1, m, dtype=np.uint64, endpoint=True)
    K[:50] = np.arange(50, dtype=np.uint64)                # u ~ 0
    K[50:100] = np.uint64(2**64 - 1) - np.arange(50, dtype=np.uint64)  # u rounds to 1: clamped
    u = np.minimum(K.astype(np.float64) * 2.0 ** -64, 1.0 - 2.0 ** -53)
    target = rng.integers(-128, 129, m).astype(np.float64)
    x0 = ((target - u) * scale.astype(np.float64)).astype(np.float32)
    step = rng.integers(-3, 4, m)
    x = x0.copy()
    for s in (-3, -2, -1, 1, 2, 3):
        sel = step == s
        x[sel] = np.nextafter(x0[sel], np.float32(np.sign(s) * np.inf), dtype=np.float32)
        for _ in range(abs(s) - 1):
            x[sel] = np.nextafter(x[sel], np.float32(np.sign(s) * np.inf), dtype=np.float32)
    # exact hits: x / scale an integer, u ~ 0 or clamped just below 1
    scale[:100] = np.float32(0.5)
    x[:50] = (target[:50] * 0.5).astype(np.float32)
    x[50:100] = ((target[50:100] - 1.0) * 0.5).astype(np.float32)
    # and plain random draws
    xr = rng.uniform(-130, 130, m).astype(np.float32) * scale
    X = np.concatenate([x, xr]).astype(np.float32)
    S = np.concatenate([scale, scale])
    KK = np.concatenate([K, K[::-1]])
    want = np.floor(X.astype(np.float64) / S.astype(np.float64) +
                    np.minimum(KK.astype(np.float64) * 2.0 ** -64, 1.0 - 2.0 ** -53)).astype(np.int64)
    dx, ds = torch.from_numpy(X).cuda(), torch.from_numpy(S).cuda()
    dk = torch.from_numpy(KK.view(np.int64)).cuda()
    out = torch.empty(len(X), dtype=torch.int32, device="cuda")
    und = torch.empty(len(X), dtype=torch.uint8, device="cuda")
    lib = N.load()
    N.check(lib.qg_dither_floor_pairs(C.c_void_p(dx.data_ptr()), C.c_void_p(ds.data_ptr()),
                                      C.c_void_p(dk.data_ptr()), len(X), C.c_void_p(out.data_ptr()),
                                      C.c_void_p(und.data_ptr()), None), "qg_dither_floor_pairs")
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.int64), want)
    u8 = und.cpu().numpy()
    assert u8[:m].sum() > 0, "boundary cases must reach the double fallback"
    assert u8[m:].sum() <= 2, "random draws should be decided in FP32"


def test_prepare_query_norm_fallbacks(cuda, oracle):
    """||q - c||^2 in the exact fixed-point path and its double-chain fallback: a float tie,
    a denormal result, a query on the centre, and wide dynamic ranges."""
    torch = cuda
    dim = 96
    c = np.zeros(dim, np.float32)
    rng = np.random.default_rng(5)
    Q = np.zeros((8, dim), np.float32)
    Q[0, 0] = np.float32(1.0 + 2.0 ** -12)      # q0^2 = 1 + 2^-11 + 2^-24: a float tie
    Q[1, 5] = np.float32(1e-20)                   # ||q||^2 below the float normal range
    Q[2] = rng.standard_normal(dim) * np.float32(1e-12)
    Q[3] = (rng.standard_normal(dim) * np.exp(rng.uniform(-30, 30, dim))).astype(np.float32)
    Q[4] = rng.standard_normal(dim) * np.float32(1e15)
    Q[5, ::2] = 1.0
    Q[5, 1::2] = -1.0
    Q[6] = rng.standard_normal(dim)
    o = oracle.Oracle(dim, c)
    sp = _space(torch, dim, c)
    p = sp.prepare(torch.from_numpy(Q).cuda())
    c2 = (rng.standard_normal(dim)).astype(np.float32)
    Q2 = np.stack([c2, c2 + np.float32(1e-6), -c2, c2 * np.float32(3.0)]).astype(np.float32)
    o2 = oracle.Oracle(dim, c2)
    sp2 = _space(torch, dim, c2)
    p2 = sp2.prepare(torch.from_numpy(Q2).cuda())
    for pp, oo, QQ in ((p, o, Q), (p2, o2, Q2)):
        for i in range(len(QQ)):
            po = oo.prepare(QQ[i])
            sc = pp["scalars"][i].cpu().numpy()
            np.testing.assert_array_equal(bits(sc), bits(np.array([po["query_norm_sqr"], po["query_norm"],
                                                                   po["half_sum"], po["scale"]], np.float32)))
            np.testing.assert_array_equal(pp["codes"][i].cpu().numpy(), po["codes"])



def test_round_quotient_decision_near_half_integers(cuda):
    """The encoder's FP32 rounding of x / s equals clamp(round(double(x)/double(s)), -7, 7),
    including quotients on and a few ulps around half-integers (where it must fall back)."""
    torch = cuda
    import ctypes as C

    from quantization_graph_gb300 import _native as N

    rng = np.random.default_rng(12)
    m = 20000
    s = rng.uniform(1e-4, 2.0, m).astype(np.float32)
    half = rng.integers(-8, 8, m) + 0.5
    x0 = (half * s.astype(np.float64)).astype(np.float32)
    x = x0.copy()
    step = rng.integers(-3, 4, m)
    for k in (-3, -2, -1, 1, 2, 3):
        sel = step == k
        for _ in range(abs(k)):
            x[sel] = np.nextafter(x[sel], np.float32(np.sign(k) * np.inf), dtype=np.float32)
    s[:200] = np.float32(0.25)                      # exact half-integers: ties away from zero
    x[:200] = (half[:200] * 0.25).astype(np.float32)
    xr = (rng.standard_normal(m) * 4).astype(np.float32) * s
    X = np.concatenate([x, xr]).astype(np.float32)
    S = np.concatenate([s, s])
    q = X.astype(np.float64) / S.astype(np.float64)
    aq = np.abs(q)
    fl = np.floor(aq)
    want = np.clip(np.sign(q) * (fl + (aq - fl >= 0.5)), -7, 7).astype(np.int64)  # C round(), exactly
    dx, ds = torch.from_numpy(X).cuda(), torch.from_numpy(S).cuda()
    out = torch.empty(len(X), dtype=torch.int32, device="cuda")
    und = torch.empty(len(X), dtype=torch.uint8, device="cuda")
    lib = N.load()
    N.check(lib.qg_round_quotient_pairs(C.c_void_p(dx.data_ptr()), C.c_void_p(ds.data_ptr()), len(X),
                                        C.c_void_p(out.data_ptr()), C.c_void_p(und.data_ptr()), None),
            "qg_round_quotient_pairs")
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.int64), want)
    u8 = und.cpu().numpy()
    assert u8[:200].sum() > 0
    assert u8[m:].sum() <= 2


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d1536"])
def test_b1_codec_prepare_and_gate_bit_exact(cuda, name):
    """The B1 query codec on the GPU: sign bits (in the code buffer), the 1-bit estimator's
    scales (short scale in the scale slot, error scale and alpha packed in the code-sum slot)
    and the popcount gate against the reference with codec 1."""
    torch = cuda
    g = load_golden(name)
    v = load_golden("b1_codec")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    sp = _space(torch, dim, g["center"], codec=1)
    p = sp.prepare(torch.from_numpy(Q).cuda())
    D = sp.code_dim
    np.testing.assert_array_equal(p["codes"].cpu().numpy().view(np.uint8)[:, :D // 8], v[f"{name}_bits"])
    sc = p["scalars"].cpu().numpy()
    packed = p["code_sum"].cpu().numpy().view(np.uint32).reshape(nq, 2)
    np.testing.assert_array_equal(bits(sc[:, 3]), bits(v[f"{name}_scalars"][:, 0]))
    np.testing.assert_array_equal(packed[:, 0], bits(v[f"{name}_scalars"][:, 1]))
    np.testing.assert_array_equal(packed[:, 1], bits(v[f"{name}_scalars"][:, 2]))
    qidx = np.repeat(np.arange(nq), n).astype(np.int32)
    ids = np.tile(np.arange(n), nq).astype(np.int32)
    gate = sp.gate_pairs(p, qidx, ids, torch.from_numpy(g["msb"]).cuda(), torch.from_numpy(g["factors"]).cuda(),
                         1.9).cpu().numpy()
    np.testing.assert_array_equal(gate[:, :21], v[f"{name}_gate"].reshape(nq * n, -1)[:, :21])
