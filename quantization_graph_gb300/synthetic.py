"""Seeded synthetic stand-ins for the reference's datasets, with the shapes and value
distributions of the workloads the reference is measured on (DBpedia-1M 1536-d, GIST-1M
960-d, AGNews 1024-d are not available offline).

  gmm          -- k-component Gaussian mixture, centres N(0,1), per-component sigma
  anisotropic  -- x ~ N(0, Q diag(lambda) Q^T), lambda_i proportional to i^-alpha, Q a seeded
                  random orthogonal matrix; optional |x| (960-d workload) or L2 normalisation
                  (1536-d workload)
  clustered    -- mixture of anisotropic Gaussians: centres N(0, (sum(lambda)/d) I) (between-
                  and within-cluster variance equal), within cluster c N(0, Q_c diag(lambda)
                  Q_c^T) with its own rotation, then L2-normalised (1024-d streaming workload)

numpy versions are bit-reproducible on every host (used by fixtures and tests); the torch
versions generate large sets directly on the GPU for the benchmark.
"""
from __future__ import annotations

import numpy as np


def gmm(n: int, dim: int, components: int = 64, sigma: float = 0.3, seed: int = 0,
        centres: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    if centres is None:
        centres = rng.standard_normal((components, dim)).astype(np.float32)
    labels = rng.integers(0, centres.shape[0], n)
    x = centres[labels] + sigma * rng.standard_normal((n, dim)).astype(np.float32)
    return x.astype(np.float32), centres


def orthogonal(dim: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((dim, dim))
    q, r = np.linalg.qr(a)
    return (q * np.sign(np.diag(r))).astype(np.float64)


def anisotropic(n: int, dim: int, alpha: float, seed: int, rotation_seed: int = 7,
                absolute: bool = False, normalize: bool = False) -> np.ndarray:
    rng = np.random.default_rng(seed)
    lam = np.arange(1, dim + 1, dtype=np.float64) ** (-alpha)
    q = orthogonal(dim, rotation_seed)
    z = rng.standard_normal((n, dim)) * np.sqrt(lam)
    x = z @ q.T
    if absolute:
        x = np.abs(x)
    if normalize:
        x /= np.maximum(np.linalg.norm(x, axis=1, keepdims=True), 1e-30)
    return x.astype(np.float32)


def anisotropic_torch(n: int, dim: int, alpha: float, seed: int, rotation_seed: int = 7,
                      absolute: bool = False, normalize: bool = False, device: str = "cuda",
                      chunk: int = 262_144):
    """GPU version of `anisotropic` for million-row sets (same law, torch RNG)."""
    import torch

    q = torch.from_numpy(orthogonal(dim, rotation_seed)).to(device=device, dtype=torch.float32)
    lam = torch.arange(1, dim + 1, device=device, dtype=torch.float64).pow(-alpha).sqrt().to(torch.float32)
    m = (q * lam[None, :]).T.contiguous()  # x = (z * sqrt(lam)) @ Q^T
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = torch.empty((n, dim), device=device, dtype=torch.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        z = torch.randn((e - s, dim), generator=g, device=device, dtype=torch.float32)
        x = z @ m
        if absolute:
            x = x.abs()
        if normalize:
            x = x / x.norm(dim=1, keepdim=True).clamp_min(1e-30)
        out[s:e] = x
    return out


def clustered_torch(n: int, dim: int, clusters: int, alpha: float, seed: int, structure_seed: int = 17,
                    device: str = "cuda", chunk: int = 131_072):
    """Unit-norm rows of a `clusters`-component mixture; cluster c has covariance
    Q_c diag(i^-alpha) Q_c^T and centre N(0, (sum_i i^-alpha / dim) I), so the spread of the
    centres equals the spread inside a cluster. The centres and rotations depend on
    `structure_seed` only, so base and query sets drawn with different `seed` share the
    mixture."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(structure_seed)
    lam64 = torch.arange(1, dim + 1, device=device, dtype=torch.float64).pow(-alpha)
    centres = torch.randn((clusters, dim), generator=g, device=device, dtype=torch.float32)
    centres *= float((lam64.sum() / dim).sqrt())
    lam = lam64.sqrt().to(torch.float32)
    mats = []
    for c in range(clusters):
        a = torch.randn((dim, dim), generator=g, device=device, dtype=torch.float32)
        qm, r = torch.linalg.qr(a)
        qm = qm * torch.sign(torch.diagonal(r))[None, :]
        mats.append((qm * lam[None, :]).T.contiguous())
    gd = torch.Generator(device=device)
    gd.manual_seed(seed)
    labels = torch.randint(0, clusters, (n,), generator=gd, device=device)
    out = torch.empty((n, dim), device=device, dtype=torch.float32)
    for c in range(clusters):
        idx = torch.nonzero(labels == c).squeeze(1)
        for s in range(0, idx.numel(), chunk):
            part = idx[s:s + chunk]
            z = torch.randn((part.numel(), dim), generator=gd, device=device, dtype=torch.float32)
            out[part] = centres[c][None, :] + z @ mats[c]
    return out / out.norm(dim=1, keepdim=True).clamp_min(1e-30)
