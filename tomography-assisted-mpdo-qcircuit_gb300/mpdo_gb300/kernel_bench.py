"""Single-kernel measurements through the public Chain API (no counterpart in
the reference).

    python -m mpdo_gb300.kernel_bench kraus1q [--l 256 --a 16 --r 256 --K 8 --reps 20 --dtype complex64]

times the Kraus application ``k_kraus1q`` on a site whose input and output
together exceed the 129 MB L2 by the engine's per-class CUDA-event profile and
prints one JSON line: launches, mean launch time, algorithmic bytes per launch
(input + output elements x element size) and the achieved GB/s.

    python -m mpdo_gb300.kernel_bench bjacobi [--m 256 --ncols 8192 --keep 64 --reps 5 --batch 24] [--split-only]

times the wide-bond block Jacobi both ways (option ``bjacobi_fused``: one
thread-block-cluster launch per eigen-solve, or one launch per tournament
round with a host read of the rotation flag per sweep) on a wide split of
that shape, on one evolution of the n=32, depth-20, chi=64, kappa=4 circuit
and on a batch of that many such circuits (seeds 0..) (``--split-only``: the
split alone), and prints one JSON line per mode.
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def kraus1q(l: int = 256, a: int = 16, r: int = 256, K: int = 8, reps: int = 20, dtype: str = 'complex64') -> dict:
    from . import build
    build()
    from .engine import Chain, Engine
    eng = Engine(0)
    eng.set_option('defer_1q', 0)          # apply at once: the launch is what is timed
    g = np.random.default_rng(0)
    site = (g.normal(size=(l, 2, a, r)) + 1j * g.normal(size=(l, 2, a, r))).astype(np.complex128)
    kr = (g.normal(size=(2, 2, K)) + 1j * g.normal(size=(2, 2, K))).astype(np.complex128)
    ch = Chain([[1, 0]] * 3, dtype=dtype, connected=True, engine=eng)
    ch.write_site(0, np.ones((1, 2, 1, l)))
    ch.write_site(2, np.ones((r, 2, 1, 1)))
    esz = 8 if dtype == 'complex64' else 16
    for k in range(reps + 2):
        ch.write_site(1, site)
        if k == 2:
            eng.sync()
            eng.profile(True)
        ch.apply_1q(1, kr)
    eng.sync()
    p = eng.profile_read()['kraus1q']
    eng.profile(False)
    per = (l * 2 * a * r) * (1 + K) * esz
    ms = p['ms'] / max(1, p['launches'])
    return {'kernel': 'k_kraus1q', 'dtype': dtype, 'site': [l, 2, a, r], 'K': K, 'launches': p['launches'],
            'mean_launch_us': 1e3 * ms, 'bytes_per_launch': per, 'achieved_gbs': per / (ms / 1e3) / 1e9}


def bjacobi(m: int = 256, ncols: int = 8192, keep: int = 64, reps: int = 5, batch: int = 24,
            dtype: str = 'complex64', split_only: bool = False):
    import time
    import torch
    from . import build
    build()
    from .engine import Batch, Chain, Engine
    from .workloads import build_circuit, u3_brickwork
    g = np.random.default_rng(1)
    y = g.normal(size=(m, ncols)) + 1j * g.normal(size=(m, ncols))
    eng = Engine(0)
    cdt = torch.complex64 if dtype == 'complex64' else torch.complex128
    if split_only:
        batch = 0
    works = [] if split_only else [u3_brickwork(n=32, depth=20, chi=64, kappa=4, seed=s) for s in range(max(batch, 1))]
    ops = [build_circuit(w, dtype=cdt, device='cuda:0')._engine_ops() for w in works]

    def evolve(k):
        w = works[k]
        ch = Chain([[1, 0]] * w.n, dtype=dtype, connected=True, engine=eng)
        for op in ops[k]:
            if op[0] == '1q':
                ch.apply_1q(op[1], op[2])
            elif op[0] == '2q':
                ch.apply_2q(op[1], op[2], 2.718281828459045e-8)
            elif op[0] == 'truncate':
                ch.truncate(w.chi, w.kappa, None, True)
            else:
                ch.kappa_truncate(w.kappa, None)
        eng.sync()
        return ch
    progs = [dict(n=w.n, dtype=dtype, vectors=[[1, 0]] * w.n, connected=True, chi=w.chi, kappa=w.kappa,
                  max_err=None, noisy=True, ops=o, z=True) for w, o in zip(works, ops)]
    bt = Batch.get(0, batch) if batch > 0 else None
    out, zs = [], {}
    try:
        for fused in (1, 0):
            eng.set_option('bjacobi_fused', fused)
            eng.debug_split(y, keep, dtype)                       # warm-up
            eng.sync()
            eng.profile(True)
            t0 = time.perf_counter()
            for _ in range(reps):
                eng.debug_split(y, keep, dtype)
            eng.sync()
            split_s = (time.perf_counter() - t0) / reps
            p = eng.profile_read()['bjacobi']
            eng.profile(False)
            rec = {'kernel': 'bjacobi', 'fused': fused, 'dtype': dtype, 'split': [m, ncols, keep],
                   'split_ms': 1e3 * split_s, 'split_bjacobi_launches': p['launches'] / reps,
                   'split_bjacobi_ms': p['ms'] / reps}
            if not split_only:
                evolve(0)                                         # warm-up
                eng.profile(True)
                t0 = time.perf_counter()
                ch = evolve(0)
                ev_s = time.perf_counter() - t0
                pe = eng.profile_read()
                eng.profile(False)
                del ch
                rec.update(evolution_s=ev_s, evolution_bjacobi_launches=pe['bjacobi']['launches'],
                           evolution_bjacobi_ms=pe['bjacobi']['ms'], evolution_wide_svd_ms=pe['phases']['wide_svd']['ms'])
            if bt is not None:
                bt.set_option('bjacobi_fused', fused)
                bt.run(progs)                                     # warm-up
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                res = bt.run(progs)
                torch.cuda.synchronize()
                bs_ = time.perf_counter() - t0
                gates = sum(sum(1 for op in o if op[0] in ('1q', '2q')) for o in ops)
                rec.update(batch=batch, batch_s=bs_, batch_gates_per_s=gates / bs_)
                zs[fused] = np.concatenate([np.asarray(r['z']) for r in res])
            out.append(rec)
    finally:
        eng.set_option('bjacobi_fused', 1)
        if bt is not None:
            bt.set_option('bjacobi_fused', 1)
    if bt is not None:
        out[-1]['batch_z_max_diff_between_modes'] = float(np.abs(zs[1] - zs[0]).max())
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('kernel', choices=['kraus1q', 'bjacobi'])
    ap.add_argument('--l', type=int, default=256)
    ap.add_argument('--a', type=int, default=16)
    ap.add_argument('--r', type=int, default=256)
    ap.add_argument('--K', type=int, default=8)
    ap.add_argument('--reps', type=int, default=None, help='default 20 (kraus1q), 5 (bjacobi)')
    ap.add_argument('--dtype', default='complex64')
    ap.add_argument('--m', type=int, default=256)
    ap.add_argument('--ncols', type=int, default=8192)
    ap.add_argument('--keep', type=int, default=64)
    ap.add_argument('--batch', type=int, default=24)
    ap.add_argument('--split-only', action='store_true', help='bjacobi: time the wide split only')
    a = ap.parse_args()
    if a.kernel == 'kraus1q':
        print(json.dumps(kraus1q(a.l, a.a, a.r, a.K, a.reps or 20, a.dtype)))
    else:
        for rec in bjacobi(a.m, a.ncols, a.keep, a.reps or 5, a.batch, a.dtype, a.split_only):
            print(json.dumps(rec), flush=True)


if __name__ == '__main__':
    main()
