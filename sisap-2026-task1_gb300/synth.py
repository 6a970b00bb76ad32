"""Seeded Gaussian-mixture datasets that stand in for the SISAP WIKIPEDIA set.

The SISAP 2026 Task 1 benchmark (6.35M x 1024 bge-m3 embeddings) is not
available offline, so every workload is synthetic with its shape:
  * C centres drawn from N(0, I_d) and normalised to unit length;
  * each point picks a centre with probability p_j proportional to j**-1.1
    (Zipf s = 1.1, so cluster sizes are multinomial with those weights and the
    ids are in random order with respect to the clusters);
  * x = centre + N(0, 0.35**2 / d * I), then L2-normalised; float32 rows.
All arithmetic is float64 numpy with a PCG64 generator, then cast to float32,
so the same (n, d, centres, seed) gives the same bytes on every host.
``mixture_torch`` draws the same kind of data on a CUDA device for sizes that
numpy would take minutes over (it is a different stream of random numbers): the
cluster labels come from numpy's PCG64 on the host and the centres and noise
from torch's seeded CUDA generator, so the same arguments give the same bytes in
every process on the same GPU type (torch.multinomial over tens of thousands of
categories on CUDA did not: its rows differed from process to process).
"""
from __future__ import annotations

import numpy as np

NOISE = 0.35
ZIPF_S = 1.1


def zipf_weights(centres: int) -> np.ndarray:
    w = np.arange(1, centres + 1, dtype=np.float64) ** -ZIPF_S
    return w / w.sum()


def mixture(n: int, d: int, centres: int, seed: int, chunk: int = 65536) -> np.ndarray:
    """Return an (n, d) float32 array of unit rows from the seeded mixture."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.standard_normal((centres, d))
    c /= np.sqrt(np.sum(c * c, axis=1, keepdims=True))
    labels = rng.choice(centres, size=n, p=zipf_weights(centres))
    out = np.empty((n, d), dtype=np.float32)
    sigma = NOISE / np.sqrt(d)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        x = c[labels[s:e]] + sigma * rng.standard_normal((e - s, d))
        x /= np.sqrt(np.sum(x * x, axis=1, keepdims=True))
        out[s:e] = x
    return out


def mixture_torch(n: int, d: int, centres: int, seed: int, device="cuda", chunk: int = 1 << 20):
    """Same distribution as ``mixture`` drawn with torch on ``device``."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    c = torch.randn(centres, d, generator=g, device=device, dtype=torch.float32)
    c /= c.norm(dim=1, keepdim=True)
    labels = np.random.Generator(np.random.PCG64(seed)).choice(centres, size=n, p=zipf_weights(centres))
    out = torch.empty(n, d, device=device, dtype=torch.float32)
    sigma = NOISE / d ** 0.5
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        lab = torch.from_numpy(labels[s:e]).to(device)
        x = c[lab] + sigma * torch.randn(e - s, d, generator=g, device=device)
        out[s:e] = x / x.norm(dim=1, keepdim=True)
    return out


def subspace(n: int, d: int, m: int, seed: int, chunk: int = 65536) -> np.ndarray:
    """(n, d) float32 unit rows spread over a random m-dimensional subspace.

    x = normalise(z A) with z ~ N(0, I_m) per row and one Gaussian m x d basis
    A: data of low intrinsic dimension, like embeddings whose spectrum decays
    fast.  Here the int8 codes keep the neighbour order well enough that the
    reference algorithm reaches recall@15 in the reference's published range
    (m = 64, 100k rows: about 84 % in 7 iterations), so recall differences of
    half a point are measurable -- unlike the isotropic mixture, where every
    method sits near 30-45 %.  float64 numpy with PCG64, cast to float32.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.standard_normal((m, d))
    out = np.empty((n, d), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        x = rng.standard_normal((e - s, m)) @ a
        x /= np.sqrt(np.sum(x * x, axis=1, keepdims=True))
        out[s:e] = x
    return out


def exact_knn(x: np.ndarray, k: int, rows=None, block: int = 2048) -> np.ndarray:
    """Exact top-k neighbours (0-based ids, self excluded) by float64 inner product.

    A float32 pass keeps the best k + 48 candidates per row, which are then
    rescored in float64.  ``rows`` restricts the queries to a subset.
    """
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    x64 = x32.astype(np.float64)
    q = np.arange(x.shape[0]) if rows is None else np.asarray(rows)
    out = np.empty((len(q), k), dtype=np.int64)
    m = min(k + 48, x.shape[0] - 1)
    for s in range(0, len(q), block):
        qi = q[s:s + block]
        sims = x32[qi] @ x32.T
        sims[np.arange(len(qi)), qi] = -np.inf
        cand = np.argpartition(-sims, m - 1, axis=1)[:, :m]
        exact = np.einsum("bd,bmd->bm", x64[qi], x64[cand])
        exact[cand == qi[:, None]] = -np.inf
        order = np.lexsort((cand, -exact), axis=1)[:, :k]
        out[s:s + block] = np.take_along_axis(cand, order, axis=1)
    return out


def recall_at_k(pred_knns_1based: np.ndarray, gt: np.ndarray, rows=None) -> float:
    """Recall as scripts/evaluation/evaluate_submission.py:18-26 defines it.

    ``pred_knns_1based`` is the exported (n, k) matrix (1-based ids); ``gt`` holds
    0-based exact neighbours of the same rows (self already excluded).
    """
    pred = np.asarray(pred_knns_1based)
    if rows is not None:
        pred = pred[np.asarray(rows)]
    k = pred.shape[1]
    hits = 0
    for p, g in zip(pred - 1, gt[:, :k]):
        hits += len(np.intersect1d(p, g))
    return hits / (pred.shape[0] * k)
