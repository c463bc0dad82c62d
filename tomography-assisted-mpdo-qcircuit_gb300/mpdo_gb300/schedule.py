"""Cost estimates of circuits and their cost-balanced split over GPUs.

The estimate is the flop count of the reference's algorithm on the circuit,
from its shape trace (host arithmetic only): per 1q gate the Kraus
contraction, per 2q gate the two-site contraction, the gate mix and the thin
SVD of theta; per truncate the QR of every site with R absorbed, the thin SVD
of every contracted pair of the right-to-left sweep and the kappa SVDs
(Circuit.py:74-178, 469-491; TNNOptimizer.py:87-197).  Contraction
M x N x K: 8 M N K; Householder QR m x n (m >= n): 4 (4 m n^2 - 4 n^3 / 3);
thin SVD m x n (m >= n): 4 (4 m n^2 + 22 n^3).  The split keeps
min(rows, cols) values (the reference's cutoff only drops a tail under
2.7e-8).  It also orders work inside one GPU's batch (longest first).

``partition`` splits independent circuits over ranks so that the estimated
work per rank is even (longest processing time first: each circuit, in
descending cost, goes to the rank with the least work so far).  Circuits are
independent, so the split needs no collective on the data path.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def _qr_flops(m: int, n: int) -> float:
    m, n = max(m, n), min(m, n)
    return 4.0 * (4.0 * m * n * n - 4.0 * n ** 3 / 3)


def _svd_flops(m: int, n: int) -> float:
    m, n = max(m, n), min(m, n)
    return 4.0 * (4.0 * m * n * n + 22.0 * n ** 3)


def reference_flops(w, K1: int = 8, K2: int = 16) -> Tuple[float, List[float]]:
    """(total, per truncate layer) flops of the reference's algorithm on the
    workload ``w`` (``mpdo_gb300.workloads.Workload``); K1 / K2 are the Kraus
    ranks of the 1q and 2q noise channels."""
    n = w.n
    l, a, r = [1] * n, [1] * n, [1] * n
    total, per_layer, cur = 0.0, [], 0.0
    for L in w.layers:
        if L[0] == '1q':
            q = L[3]
            cur += 8.0 * 2 * K1 * 2 * l[q] * a[q] * r[q]
            a[q] *= K1
        elif L[0] == '2q':
            i = min(L[3], L[4])
            m = r[i]
            rows, cols = l[i] * 2 * a[i], 2 * a[i + 1] * K2 * r[i + 1]
            cur += 8.0 * rows * (2 * a[i + 1] * r[i + 1]) * m + 8.0 * 4 * K2 * 4 * l[i] * a[i] * a[i + 1] * r[i + 1]
            cur += _svd_flops(rows, cols)
            keep = min(rows, cols)
            r[i] = l[i + 1] = keep
            a[i + 1] *= K2
        else:
            for i in range(n - 1):                                   # QR sweep
                mm, nn = l[i] * 2 * a[i], r[i]
                k = min(mm, nn)
                cur += _qr_flops(mm, nn) + 8.0 * k * nn * 2 * a[i + 1] * r[i + 1]
                r[i] = l[i + 1] = k
            for idx in range(n - 1, 0, -1):                          # SVD sweep on contracted pairs
                rows, cols = l[idx - 1] * 2 * a[idx - 1], 2 * a[idx] * r[idx]
                cur += 8.0 * rows * cols * r[idx - 1] + _svd_flops(rows, cols)
                keep = min(w.chi, rows, cols)
                r[idx - 1] = l[idx] = keep
            for i in range(n):                                       # kappa pass
                if a[i] > w.kappa:
                    cur += _svd_flops(l[i] * 2 * r[i], a[i])
                    a[i] = min(w.kappa, l[i] * 2 * r[i], a[i])
            per_layer.append(cur)
            total += cur
            cur = 0.0
    return total + cur, per_layer


def partition(costs: Sequence[float], ranks: int) -> List[List[int]]:
    """Indices of ``costs`` split over ``ranks`` parts by longest processing
    time first (ties by index, so every rank computes the same split).  Each
    part lists its circuits in descending cost."""
    if ranks < 1:
        raise ValueError('ranks must be >= 1')
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    parts: List[List[int]] = [[] for _ in range(ranks)]
    load = [0.0] * ranks
    for i in order:
        r = min(range(ranks), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    return parts


def imbalance(parts: Sequence[Sequence[int]], costs: Sequence[float]) -> float:
    """Largest part's estimated work over the mean part's (1.0 = even)."""
    loads = [sum(float(costs[i]) for i in p) for p in parts]
    mean = sum(loads) / len(loads) if loads else 0.0
    return max(loads) / mean if mean > 0 else 1.0
