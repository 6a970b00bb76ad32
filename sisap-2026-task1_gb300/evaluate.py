"""Ground truth and recall for kNN-graph outputs (GPU), after the reference's
scripts/evaluation/evaluate_submission.py.

    python evaluate.py GT.h5 PRED.h5
        recall = sum_i |pred_i ∩ (gt_i without i+1)[:k]| / (n * k), with gt =
        /allknn/knns (1-based) and pred = knns, as evaluate_submission.py:18-26.
    python evaluate.py --ground-truth DATA.h5 GT.h5 [--k 32]
        exact all-points k-NN of /train by inner product, written as
        /allknn/knns (1-based, self included first, like the benchmark's files)
        and /allknn/dists.

Ground truth on the GPU: a tensor-core pass (TF32) keeps the best k + 64
candidates of every row, which are rescored in float64 and ordered by (score
desc, id asc).  Files are knng containers (see h5container.py).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import h5container  # noqa: E402


def all_knn(x, k=32, block=2048, margin=64):
    """Exact top-k (including self) of every row of x (torch CUDA float32, unit or
    not) by float64 inner product; returns (ids int64 [n, k] 0-based, scores f64)."""
    import torch

    n = x.shape[0]
    m = min(n, k + margin)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    ids = torch.empty((n, k), dtype=torch.int64, device=x.device)
    sc = torch.empty((n, k), dtype=torch.float64, device=x.device)
    try:
        for s in range(0, n, block):
            q = x[s:s + block]
            cand = (q @ x.T).topk(m, dim=1).indices
            exact = torch.einsum("bd,bmd->bm", q.double(), x[cand].double())
            # order by (score desc, id asc): sort ids first, then a stable sort on score
            o1 = cand.argsort(dim=1)
            cand = torch.gather(cand, 1, o1)
            exact = torch.gather(exact, 1, o1)
            o2 = exact.argsort(dim=1, descending=True, stable=True)[:, :k]
            ids[s:s + block] = torch.gather(cand, 1, o2)
            sc[s:s + block] = torch.gather(exact, 1, o2)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return ids, sc


def sample_knn(x, rows, k=15, block=500, margin=64):
    """Exact top-k neighbours, self excluded, of the given rows of x (torch CUDA
    float32 [n, d]) by float64 inner product: a float32 pass keeps the best
    k + margin candidates, which are rescored in float64 and ordered by (score
    desc, candidate position).  Returns 0-based ids as numpy int64 [len(rows), k]."""
    import torch

    rows = torch.as_tensor(np.asarray(rows), device=x.device)
    m = min(x.shape[0] - 1, k + margin)
    out = []
    for s in range(0, len(rows), block):
        q = rows[s:s + block]
        sims = x[q] @ x.T
        sims[torch.arange(len(q), device=x.device), q] = -float("inf")
        cand = sims.topk(m, dim=1).indices
        del sims
        exact = torch.einsum("bd,bmd->bm", x[q].double(), x[cand].double())
        exact[cand == q[:, None]] = -float("inf")
        order = exact.argsort(dim=1, descending=True, stable=True)[:, :k]
        out.append(torch.gather(cand, 1, order).cpu())
    return torch.cat(out).numpy()


def recall(gt_knns_1based, pred_knns_1based):
    """evaluate_submission.py:17-26: per row, the first k gt ids other than the
    row itself, intersected with the row's predicted ids."""
    gt = np.asarray(gt_knns_1based)
    pred = np.asarray(pred_knns_1based)
    n, k = pred.shape
    hits = 0
    for i in range(n):
        g = gt[i][gt[i] != (i + 1)][:k]
        hits += len(np.intersect1d(pred[i], g))
    return hits / (n * k)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("files", nargs=2)
    ap.add_argument("--ground-truth", action="store_true")
    ap.add_argument("--k", type=int, default=32)
    a = ap.parse_args(argv)
    if a.ground_truth:
        import torch

        ds, _ = h5container.read(a.files[0])
        x = torch.from_numpy(np.asarray(ds["train"], dtype=np.float32)).cuda()
        ids, sc = all_knn(x, a.k)
        h5container.write(a.files[1], {"allknn/knns": (ids + 1).to(torch.int32).cpu().numpy(),
                                       "allknn/dists": sc.float().cpu().numpy()})
        print(f"wrote exact {a.k}-NN of {x.shape[0]} rows to {a.files[1]}")
        return 0
    gt, _ = h5container.read(a.files[0])
    pred, attrs = h5container.read(a.files[1])
    r = recall(gt["allknn/knns"], pred["knns"])
    print("==================================================")
    print(f"Algorithm:   {attrs.get('algo', 'Unknown')}")
    print(f"Vectors:     {pred['knns'].shape[0]}")
    print(f"Build Time:  {attrs.get('buildtime', 0.0)} seconds")
    print(f"True Recall: {r * 100:.4f}%")
    print("==================================================")
    return 0


if __name__ == "__main__":
    sys.exit(main())
