"""The encode rotation as a BF16x3 GEMM on the tcgen05 tensor cores (qg_rotate_gemm,
qg_encode_batch_gemm) against FP64 arithmetic and against the reference encoder.

The rotation's operands are exact (three BF16 terms of each scaled residual value, a +-1
Hadamard-sign matrix), so the GEMM may differ from the exact product only by the FP32
accumulation: at most 3 Kp * 2^-24 * sum|a| per value, whatever the summation order. Codes
from the GEMM path are compared with the reference encoder's (the FHT path, bit-exact to the
reference); they may differ only where the summation order moves a value across a boundary."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _hadamard_signs(D, dim, signs):
    i = np.arange(dim)[None, :]
    j = np.arange(D)[:, None]
    pop = np.vectorize(lambda v: bin(v).count("1"))(i & j)
    return np.where(pop & 1, -1.0, 1.0) * np.where(signs[:dim] > 0, 1.0, -1.0)[None, :]


def _scaled_rows(x, center, c_abs):
    """The split kernel's a = fl(fl(r * (1 / |r|)) * c) in float32, |r| by a sequential float32 sum."""
    r = (x - center[None, :]).astype(np.float32)
    rns = np.cumsum(r * r, axis=1, dtype=np.float32)[:, -1]
    rn = np.sqrt(rns).astype(np.float32)
    inv = (np.float32(1.0) / rn).astype(np.float32)
    u = np.where(rn[:, None] > 0, (r * inv[:, None]).astype(np.float32), r)
    return (u * np.float32(c_abs)).astype(np.float32), rn


@pytest.mark.parametrize("dim,n", [(1536, 300), (960, 129), (200, 64)])
def test_rotation_gemm_within_the_fp32_accumulation_bound(cuda, dim, n):
    torch = cuda
    from quantization_graph_gb300.space import RabitqSpace

    rng = np.random.default_rng(dim)
    x = rng.standard_normal((n, dim)).astype(np.float32)
    center = rng.standard_normal(dim).astype(np.float32) * 0.1
    x[3] = center  # a row on the centre: zero residual
    sp = RabitqSpace(dim, center)
    D = sp.code_dim
    rot, norms = sp.rotate_gemm(torch.from_numpy(x))
    rot = rot.cpu().numpy().astype(np.float64)
    signs = sp.signs()
    with np.errstate(divide="ignore", invalid="ignore"):
        a, rn = _scaled_rows(x, center, abs(float(signs[0])))
    np.testing.assert_array_equal(norms.cpu().numpy(), rn)  # the encoder's own norm, bit for bit
    R = _hadamard_signs(D, dim, signs)
    exact = a.astype(np.float64) @ R.T
    kp = (dim + 63) // 64 * 64
    bound = 3 * kp * 2.0 ** -24 * np.abs(a).astype(np.float64).sum(1)[:, None] + 1e-30
    err = np.abs(rot - exact)
    assert (err <= bound).all(), float((err / bound).max())
    assert (rot[3] == 0).all()


def test_rotation_gemm_close_to_the_reference_fht(cuda, oracle):
    torch = cuda
    from quantization_graph_gb300.space import RabitqSpace

    rng = np.random.default_rng(7)
    dim, n = 1536, 64
    x = rng.standard_normal((n, dim)).astype(np.float32)
    center = rng.standard_normal(dim).astype(np.float32) * 0.1
    sp = RabitqSpace(dim, center)
    rot, norms = sp.rotate_gemm(torch.from_numpy(x))
    o = oracle.Oracle(dim, center)
    np.testing.assert_array_equal(o.signs(), sp.signs())
    rn = norms.cpu().numpy()
    for v in range(n):  # the oracle rotates u = fl(r * (1 / |r|)) by signs and butterflies
        fht = o.rotate(((x[v] - center).astype(np.float32) * (np.float32(1.0) / rn[v])).astype(np.float32))
        assert np.abs(rot[v].cpu().numpy() - fht).max() < 1e-5, v


def test_gemm_encode_matches_the_reference_encoder_but_for_rare_boundaries(cuda):
    torch = cuda
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.space import RabitqSpace

    dim, n = 1536, 3000
    x = synthetic.anisotropic(n, dim, 0.8, seed=5, normalize=True)
    center = x.mean(0).astype(np.float32)
    sp = RabitqSpace(dim, center)
    c_ref, r_ref = sp.encode(torch.from_numpy(x))       # the FHT path, bit-exact to the reference
    c_gem, r_gem = sp.encode_gemm(torch.from_numpy(x))  # the tensor-core rotation
    c_ref, c_gem = c_ref.cpu().numpy(), c_gem.cpu().numpy()
    D = sp.code_dim
    codes_r, codes_g = c_ref[:, 16:16 + D // 2], c_gem[:, 16:16 + D // 2]
    bad = ((codes_r & 15) != (codes_g & 15)).sum() + ((codes_r >> 4) != (codes_g >> 4)).sum()
    rate = bad / (n * D)
    assert rate < 1e-3, rate
    f_r = c_ref[:, :16].copy().view(np.float32).astype(np.float64)
    f_g = c_gem[:, :16].copy().view(np.float32).astype(np.float64)
    rel = np.abs(f_r - f_g) / np.maximum(np.abs(f_r), 1e-30)
    assert rel[:, 0].max() == 0.0  # norm_sqr does not depend on the rotation
    # the tensor cores' FP32 accumulation is coarser than the butterflies' rounded adds: the other
    # factors move by a few parts per million (a handful more where a code changes)
    assert np.median(rel[:, 1:]) < 2e-5 and rel[:, 1:].max() < 0.2
    print(f"code mismatch rate {rate:.2e}, records equal {(c_ref == c_gem).all(1).mean():.4f}")


def test_rotation_gemm_refuses_small_code_dims(cuda):
    torch = cuda
    from quantization_graph_gb300.space import RabitqSpace

    sp = RabitqSpace(128, np.zeros(128, np.float32))
    with pytest.raises(RuntimeError, match="QG_ERR_UNSUPPORTED"):
        sp.rotate_gemm(torch.zeros((4, 128)))


@pytest.mark.parametrize("plane", [0, 1, 2])
def test_rotation_gemm_is_exact_where_the_sums_are_representable(cuda, plane):
    """Operand planes of integers times a power of two (exact in BF16) whose every partial sum
    fits 24 bits: the GEMM must return the exact product, from any one of the three planes."""
    torch = cuda
    import ctypes as C

    from quantization_graph_gb300 import _native as N
    from quantization_graph_gb300.space import RabitqSpace, _stream

    dim, n = 1536, 200
    sp = RabitqSpace(dim, np.zeros(dim, np.float32))
    D = sp.code_dim
    kp = (dim + 63) // 64 * 64
    rng = np.random.default_rng(plane)
    ints = rng.integers(-127, 128, (n, dim)).astype(np.int64)
    scale = 2.0 ** (-7 - 8 * plane)
    a3 = np.zeros((n, 3 * kp), np.float32)
    a3[:, plane * kp:plane * kp + dim] = (ints * scale).astype(np.float32)
    bits = (a3.view(np.uint32) >> 16).astype(np.uint16)  # exact: 8 significant bits at most
    assert np.array_equal((bits.astype(np.uint32) << 16).view(np.float32), a3)
    R = _hadamard_signs(D, dim, sp.signs()).astype(np.int64)
    want = (ints @ R.T).astype(np.float64) * scale  # |sum| < 2^18 units: exact in FP32
    out = torch.empty((n, D), dtype=torch.float32, device="cuda")
    d_a3 = torch.from_numpy(bits.view(np.int16)).cuda()
    lib = N.load()
    N.check(lib.qg_rotate_gemm_planes(sp.ptr, C.c_void_p(d_a3.data_ptr()), n, C.c_void_p(out.data_ptr()), _stream()),
            "qg_rotate_gemm_planes")
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.float64), want)
