"""Generates the golden fixtures under tests/golden/ from the REFERENCE ITSELF.

Runs only on a host that has the reference tree: oracle/Makefile compiles the reference's
own experiments/02_diskann_fair/native/rabitq_bridge.cpp (with the reference's flags,
-O3 -march=native on x86-64) into oracle/_ref/libqg_ref.so. Every expected value below comes
from that library: encode (rabitq_encode_full + copy_compact / copy_residual_record), the
sidecar (rabitq_export_paper_sidecar), the INT8 prepared query (read from the reference's
PreparedQuery), the batched gate / distance / residual kernels, the Vamana graph
(rabitq_build_vamana_graph) and search results, where the Rust hot loop of
ours_diskann.rs:1539-1986 (which cannot be built here) is driven over the reference's own
bridge kernels (oracle/ref_probe.cpp).

Inputs are regenerated from numpy seeds in the tests; a checksum of each input is stored
to catch generator drift.  Usage:  python tests/golden/make_golden.py [build_variants | space_states | int4 | b1 | build_edges | b1main | full | fused | encoded_gate]
"""
from __future__ import annotations

import hashlib
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle_py  # noqa: E402
sys.path.insert(0, HERE)
from cases import BUILD_EDGE_ARGS, BUILD_VARIANTS, build_edge_data, c1_data, c2_data, c3_data, kernel_inputs  # noqa: E402

FLAGS = "g++ -std=c++20 -O3 -march=native -fopenmp (experiments/02_diskann_fair/build.rs:22-36)"


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def kernel_case(name: str, dim: int, n: int, nq: int, seed: int, center_value: float | None, codec: int = 3):
    """Kernel-level golden vectors for every query x every record (codec 3 = Int8, 2 = Int4)."""
    X, Q = kernel_inputs(dim, n, nq, seed)
    center = (np.full(dim, center_value, np.float32) if center_value is not None
              else X.mean(0).astype(np.float32))
    ref = oracle_py.Reference(dim, center, codec=codec)
    full = np.stack([ref.encode_full(x) for x in X])
    compact, residual = ref.encode(X)
    msb, factors = ref.sidecar(compact)
    ids = np.arange(n, dtype=np.uint32)
    out = dict(dim=dim, n=n, nq=nq, seed=seed, codec=codec, center=center, x_sha=sha(X), q_sha=sha(Q), full=full,
               compact=compact, residual=residual, msb=msb, factors=factors)
    rr, codes, scal, csum, gate, d2, d0, res, dsingle = [], [], [], [], [], [], [], [], []
    for q in Q:
        p = ref.prepare(q)
        rr.append(p["rotated_residual"])
        codes.append(p["codes"])
        scal.append([p["query_norm_sqr"], p["query_norm"], p["half_sum"], p["scale"]])
        csum.append(p["code_sum"])
        g = ref.gate(ids, msb, factors, 1.9)
        gate.append(g.view(np.uint8).reshape(n, -1))
        d2.append(ref.distance(ids, np.full(n, 2, np.uint8), compact, g["short_ip"]))
        dd0 = ref.distance(ids, np.zeros(n, np.uint8), compact, np.zeros(n, np.float32))
        d0.append(dd0)
        dsingle.append(np.array([ref.distance_single(compact[i]) for i in range(n)], np.float32))
        res.append(ref.residual(ids, compact, residual, dd0).view(np.float32).reshape(n, 3))
    out.update(rotated_residual=np.array(rr), codes=np.array(codes), scalars=np.array(scal, np.float32),
               code_sum=np.array(csum, np.int64), gate=np.array(gate), dist_mode2=np.array(d2),
               dist_mode0=np.array(d0), dist_single=np.array(dsingle), residual_iv=np.array(res))
    sym = np.array([[ref.symmetric_distance(compact[i], compact[j]) for j in range(min(n, 16))]
                    for i in range(min(n, 16))], np.float32)
    out["symmetric"] = sym
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, "written")


def search_case(name: str, data_fn, dim: int, n: int, nq: int, seed: int, M: int, l_build: int,
                refine: int, cap: int, stop: int, batch: int, Ls, ks=(10,), extra=None):
    X, Q = data_fn()
    center = X.mean(0).astype(np.float32)  # N <= 100k: the reference centre is the f32 mean
    ref = oracle_py.Reference(dim, center)
    compact, residual = ref.encode(X)
    deg, edges = ref.build_graph(compact, r=M, l_build=l_build, alpha=1.2, batch=batch, refine=refine,
                                 cap=cap, stop_hops=stop)
    msb, factors = ref.sidecar(compact)
    index = dict(compact=compact, residual=residual, msb=msb, factors=factors, degrees=deg, edges=edges,
                 total_points=n, base_points=n)
    orc = oracle_py.Oracle(dim, center)
    gt, gtd = orc.exact_knn(X, Q, 100)
    out = dict(dim=dim, n=n, nq=nq, seed=seed, center=center, x_sha=sha(X), q_sha=sha(Q), compact=compact,
               residual=residual, msb=msb, factors=factors, degrees=deg, edges=edges, gt=gt,
               Ls=np.array(Ls), ks=np.array(ks))
    for L in Ls:
        for k in ks:
            ids, dists, stats = ref.search(Q, index, k=k, L=L, eps=1.9, rerank=100)
            out[f"ids_L{L}_k{k}"] = ids
            out[f"dists_L{L}_k{k}"] = dists
            out[f"stats_L{L}_k{k}"] = stats.view(np.uint64).reshape(nq, -1)
            rec = np.mean([len(set(a[:10]) & set(b[:10])) / 10 for a, b in zip(ids, gt)]) if k >= 10 else -1
            print(f"  {name} L={L} k={k} recall@10={rec:.4f}")
    if extra:
        extra(out, ref, Q, index)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, "written")


def c1_extras(out, ref, Q, index):
    # beam width 2, kth stop, early stop, and k=1 / k=100 with L < k
    for tag, kw in (("beam2", dict(beam=2, L=40, k=10)), ("kth", dict(kth_stop=True, L=40, k=10)),
                    ("stall", dict(early_stop=2, L=40, k=10)), ("k100", dict(L=40, k=100)),
                    ("k1", dict(L=20, k=1))):
        ids, dists, stats = ref.search(Q, index, eps=1.9, rerank=100, **kw)
        out[f"ids_{tag}"] = ids
        out[f"dists_{tag}"] = dists
        out[f"stats_{tag}"] = stats.view(np.uint64).reshape(len(Q), -1)


def build_variants():
    """Graphs of the reference's own rabitq_build_vamana_graph for argument sets other than the
    formal one, over the records already stored in the search fixtures."""
    out = {}
    for name, kw in BUILD_VARIANTS.items():
        kw = dict(kw)
        g = np.load(os.path.join(HERE, kw.pop("src") + ".npz"))
        ref = oracle_py.Reference(int(g["dim"]), g["center"])
        deg, edges = ref.build_graph(g["compact"], **kw)
        out[f"{name}_degrees"] = deg
        out[f"{name}_edges"] = edges
        out[f"{name}_evals"] = np.array(ref.last_build_evals, np.uint64)
        print(name, "mean degree", deg.mean(), "evals", ref.last_build_evals)
    np.savez_compressed(os.path.join(HERE, "build_variants.npz"), **out)


def int4_cases():
    """The Int4 query codec (an ablation in the reference): kernel vectors for 128-d and 1536-d,
    and search results on the search_c1 index."""
    kernel_case("kernels_d128_int4", 128, 64, 8, seed=20260813, center_value=0.05, codec=2)
    kernel_case("kernels_d1536_int4", 1536, 64, 3, seed=7, center_value=None, codec=2)
    g = np.load(os.path.join(HERE, "search_c1.npz"))
    _, Q = c1_data()
    ref = oracle_py.Reference(128, g["center"], codec=2)
    index = dict(compact=g["compact"], residual=g["residual"], msb=g["msb"], factors=g["factors"],
                 degrees=g["degrees"], edges=g["edges"], total_points=int(g["n"]), base_points=int(g["n"]))
    out = {}
    for L in (20, 40, 80):
        ids, dists, stats = ref.search(Q, index, k=10, L=L, eps=1.9, rerank=100)
        out[f"ids_L{L}"] = ids
        out[f"dists_L{L}"] = dists
        out[f"stats_L{L}"] = stats.view(np.uint64).reshape(len(Q), -1)
    np.savez_compressed(os.path.join(HERE, "search_c1_int4.npz"), **out)
    print("search_c1_int4 written")


def b1main_cases():
    """The B1Main codec (no gate; every fresh neighbour by the 4-bit x 1-bit distance): the
    distance for every query x record of the kernel fixtures, and whole searches on the
    search_c1 and search_c2 indexes."""
    out = {}
    for name in ("kernels_d128", "kernels_d1536"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
        _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
        ref = oracle_py.Reference(dim, g["center"], codec=4)
        d = []
        for q in Q:
            ref.prepare(q)
            d.append([ref.distance_b1(g["compact"][i]) for i in range(n)])
        out[f"{name}_distance_b1"] = np.array(d, np.float32)
    for name, fn in (("search_c1", c1_data), ("search_c2", c2_data)):
        g = np.load(os.path.join(HERE, name + ".npz"))
        _, Q = fn()
        ref = oracle_py.Reference(int(g["dim"]), g["center"], codec=4)
        index = dict(compact=g["compact"], residual=g["residual"], msb=g["msb"], factors=g["factors"],
                     degrees=g["degrees"], edges=g["edges"], total_points=int(g["n"]), base_points=int(g["n"]))
        for L in (20, 40, 80):
            ids, dists, stats = ref.search(Q, index, k=10, L=L, eps=1.9, rerank=100)
            out[f"{name}_ids_L{L}"] = ids
            out[f"{name}_dists_L{L}"] = dists
            out[f"{name}_stats_L{L}"] = stats.view(np.uint64).reshape(len(Q), -1)
    np.savez_compressed(os.path.join(HERE, "b1main_codec.npz"), **out)
    print("b1main_codec written")


def full_cases():
    """The Full query codec (FP32 query against the MSB plane; survivors by the FP32 remaining
    bits reusing the gate's short ip, mode 1): gate and mode-1 distances for every query x record
    of three kernel fixtures, and whole searches on the three search indexes; also whole searches
    with FullRerankScalar (6), whose rerank takes the bridge's per-record residual path, and with
    FullStaged (5) and FullScalar (7), stored only where they differ from Full's."""
    out = {}
    for name in ("kernels_d128", "kernels_d960", "kernels_d1536"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
        _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
        ref = oracle_py.Reference(dim, g["center"], codec=0)
        ids = np.arange(n, dtype=np.uint32)
        gate, d1 = [], []
        for q in Q:
            ref.prepare(q)
            est = ref.gate(ids, g["msb"], g["factors"], 1.9)
            gate.append(est.view(np.uint8).reshape(n, -1))
            d1.append(ref.distance(ids, np.full(n, 1, np.uint8), g["compact"], est["short_ip"]))
        out[f"{name}_gate"] = np.array(gate)
        out[f"{name}_dist_mode1"] = np.array(d1)
    for name, fn in (("search_c1", c1_data), ("search_c2", c2_data), ("search_c3", c3_data)):
        g = np.load(os.path.join(HERE, name + ".npz"))
        _, Q = fn()
        ref = oracle_py.Reference(int(g["dim"]), g["center"], codec=0)
        index = dict(compact=g["compact"], residual=g["residual"], msb=g["msb"], factors=g["factors"],
                     degrees=g["degrees"], edges=g["edges"], total_points=int(g["n"]), base_points=int(g["n"]))
        for L in (20, 40):
            ids, dists, stats = ref.search(Q, index, k=10, L=L, eps=1.9, rerank=100)
            out[f"{name}_ids_L{L}"] = ids
            out[f"{name}_dists_L{L}"] = dists
            out[f"{name}_stats_L{L}"] = stats.view(np.uint64).reshape(len(Q), -1)
        for codec in (5, 6, 7):
            other = oracle_py.Reference(int(g["dim"]), g["center"], codec=codec)
            for L in (20, 40):
                ids, dists, stats = other.search(Q, index, k=10, L=L, eps=1.9, rerank=100)
                st = stats.view(np.uint64).reshape(len(Q), -1)
                same = (np.array_equal(ids, out[f"{name}_ids_L{L}"]) and
                        np.array_equal(dists.view(np.uint32), out[f"{name}_dists_L{L}"].view(np.uint32)) and
                        np.array_equal(st, out[f"{name}_stats_L{L}"]))
                if codec == 6 or not same:
                    out[f"{name}_c{codec}_ids_L{L}"] = ids
                    out[f"{name}_c{codec}_dists_L{L}"] = dists
                    out[f"{name}_c{codec}_stats_L{L}"] = st
    np.savez_compressed(os.path.join(HERE, "full_codec.npz"), **out)
    print("full_codec written")


def fused_rerank_cases():
    """rabitq_full_residual_distance_batch, the reference's fused FP32 restore + residual rerank
    kernel, for every query x record of three kernel fixtures, and whole Int8 / Int4 searches
    with the fused rerank switched on (RABITQ_ENABLE_FUSED_INT_RERANK) on the search indexes."""
    out = {}
    for name in ("kernels_d128", "kernels_d960", "kernels_d1536"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
        _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
        ref = oracle_py.Reference(dim, g["center"])
        ids = np.arange(n, dtype=np.uint32)
        res = []
        for q in Q:
            ref.prepare(q)
            res.append(ref.full_residual(ids, np.ascontiguousarray(g["compact"]), np.ascontiguousarray(g["residual"])))
        out[name] = np.array(res)
    for name, fn in (("search_c1", c1_data), ("search_c2", c2_data), ("search_c3", c3_data)):
        g = np.load(os.path.join(HERE, name + ".npz"))
        _, Q = fn()
        index = dict(compact=g["compact"], residual=g["residual"], msb=g["msb"], factors=g["factors"],
                     degrees=g["degrees"], edges=g["edges"], total_points=int(g["n"]), base_points=int(g["n"]))
        for codec in (3, 2):
            ref = oracle_py.Reference(int(g["dim"]), g["center"], codec=codec)
            for L in (20, 40):
                ids, dists, stats = ref.search(Q, index, k=10, L=L, eps=1.9, rerank=100, fused=True)
                out[f"{name}_c{codec}_ids_L{L}"] = ids
                out[f"{name}_c{codec}_dists_L{L}"] = dists
                out[f"{name}_c{codec}_stats_L{L}"] = stats.view(np.uint64).reshape(len(Q), -1)
    np.savez_compressed(os.path.join(HERE, "fused_rerank.npz"), **out)
    print("fused_rerank written")


def encoded_gate_cases():
    """rabitq_paper_estimate_batch (the gate from the encoded record, compute_paper_prune_estimate)
    for every query x record of four kernel fixtures, Int8 and Full prepared queries."""
    out = {}
    for name in ("kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
        _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
        ids = np.arange(n, dtype=np.uint32)
        for codec in (3, 0):
            ref = oracle_py.Reference(dim, g["center"], codec=codec)
            rows = []
            for q in Q:
                ref.prepare(q)
                rows.append(ref.gate_encoded(ids, np.ascontiguousarray(g["compact"])).view(np.uint8).reshape(n, -1))
            out[f"{name}_c{codec}"] = np.array(rows)
    np.savez_compressed(os.path.join(HERE, "encoded_gate.npz"), **out)
    print("encoded_gate written")


def build_edges():
    """Reference graphs for duplicate / near-duplicate / zero vectors and a 3-node index."""
    X = build_edge_data()
    center = X.mean(0).astype(np.float32)
    ref = oracle_py.Reference(128, center)
    compact, _ = ref.encode(X)
    out = dict(center=center, compact=compact)
    for name, kw in BUILD_EDGE_ARGS.items():
        kw = dict(kw)
        n = kw.pop("n", len(compact))
        deg, edges = ref.build_graph(compact[:n], **kw)
        out[f"{name}_degrees"] = deg
        out[f"{name}_edges"] = edges
    np.savez_compressed(os.path.join(HERE, "build_edges.npz"), **out)
    print("build_edges written")


def b1_cases():
    """The B1 query codec (sign bits; an ablation in the reference): per query the sign bits
    and the 1-bit estimator's scales, the B1 gate over every record of the kernel fixtures, and
    whole searches (survivors scored by the FP32 restore) on the search_c1 index."""
    out = {}
    for name in ("kernels_d128", "kernels_d1536"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
        _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
        ref = oracle_py.Reference(dim, g["center"], codec=1)
        ids = np.arange(n, dtype=np.uint32)
        bits, scal, ssum, gate = [], [], [], []
        for q in Q:
            p = ref.prepare(q)
            bits.append(p["b1_bits"])
            scal.append(p["b1_scalars"])
            ssum.append(p["b1_signed_sum"])
            gate.append(ref.gate(ids, g["msb"], g["factors"], 1.9).view(np.uint8).reshape(n, -1))
        out[f"{name}_bits"] = np.array(bits)
        out[f"{name}_scalars"] = np.array(scal, np.float32)
        out[f"{name}_signed_sum"] = np.array(ssum, np.int64)
        out[f"{name}_gate"] = np.array(gate)
    g = np.load(os.path.join(HERE, "search_c1.npz"))
    _, Q = c1_data()
    ref = oracle_py.Reference(128, g["center"], codec=1)
    index = dict(compact=g["compact"], residual=g["residual"], msb=g["msb"], factors=g["factors"],
                 degrees=g["degrees"], edges=g["edges"], total_points=int(g["n"]), base_points=int(g["n"]))
    for L in (20, 40, 80):
        ids, dists, stats = ref.search(Q, index, k=10, L=L, eps=1.9, rerank=100)
        out[f"search_c1_ids_L{L}"] = ids
        out[f"search_c1_dists_L{L}"] = dists
        out[f"search_c1_stats_L{L}"] = stats.view(np.uint64).reshape(len(Q), -1)
    np.savez_compressed(os.path.join(HERE, "b1_codec.npz"), **out)
    print("b1_codec written")


def space_states():
    """RaBitQSpace::saveState output of the reference for the kernel fixtures' spaces (seed 100,
    their centres): the EXRBTQ31 bytes a saved space must equal and a loaded one must encode
    like."""
    out = {}
    for name in ("kernels_d128", "kernels_d960", "kernels_d1536"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        ref = oracle_py.Reference(int(g["dim"]), g["center"])
        out[name] = np.frombuffer(ref.save_state(), np.uint8)
        print(name, "state", out[name].size, "bytes")
    np.savez_compressed(os.path.join(HERE, "space_states.npz"), **out)


def main():
    oracle_py.build(ref=True)
    if not oracle_py.reference_available():
        raise SystemExit("the reference library could not be built")
    if sys.argv[1:] == ["build_variants"]:
        build_variants()
        return
    if sys.argv[1:] == ["space_states"]:
        space_states()
        return
    if sys.argv[1:] == ["int4"]:
        int4_cases()
        return
    if sys.argv[1:] == ["b1"]:
        b1_cases()
        return
    if sys.argv[1:] == ["build_edges"]:
        build_edges()
        return
    if sys.argv[1:] == ["b1main"]:
        b1main_cases()
        return
    if sys.argv[1:] == ["full"]:
        full_cases()
        return
    if sys.argv[1:] == ["fused"]:
        fused_rerank_cases()
        return
    if sys.argv[1:] == ["encoded_gate"]:
        encoded_gate_cases()
        return
    kernel_case("kernels_d128", 128, 64, 8, seed=20260813, center_value=0.05)
    kernel_case("kernels_d100", 100, 48, 4, seed=5, center_value=None)
    kernel_case("kernels_d960", 960, 96, 4, seed=6, center_value=None)
    kernel_case("kernels_d1536", 1536, 64, 3, seed=7, center_value=None)
    # graph arguments: cases.SEARCH_GRAPH_ARGS
    search_case("search_c1", c1_data, 128, 2000, 50, 11, M=32, l_build=100, refine=1, cap=256, stop=2,
                batch=256, Ls=(20, 40, 80), extra=c1_extras)
    search_case("search_c2", c2_data, 960, 1500, 24, 21, M=32, l_build=64, refine=1, cap=256, stop=2,
                batch=256, Ls=(40, 100))
    search_case("search_c3", c3_data, 1536, 1000, 16, 31, M=32, l_build=64, refine=1, cap=256, stop=2,
                batch=256, Ls=(40,))
    build_variants()
    space_states()
    int4_cases()
    b1_cases()
    build_edges()
    b1main_cases()
    full_cases()
    fused_rerank_cases()
    encoded_gate_cases()
    with open(os.path.join(HERE, "PROVENANCE.txt"), "w") as f:
        f.write(f"generated by tests/golden/make_golden.py on {platform.machine()} {platform.processor()}\n")
        f.write(f"reference bridge compiled with: {FLAGS}\n")
        f.write("search results: the restated Rust hot loop driven over the reference bridge kernels\n")


if __name__ == "__main__":
    main()
