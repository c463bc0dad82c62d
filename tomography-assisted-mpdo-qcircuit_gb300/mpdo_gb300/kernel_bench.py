"""Single-kernel measurements through the public Chain API (no counterpart in
the reference): the Kraus application ``k_kraus1q`` on a site whose input
and output together exceed the 129 MB L2, timed by the engine's per-class
CUDA-event profile.

    python -m mpdo_gb300.kernel_bench kraus1q [--l 256 --a 16 --r 256 --K 8 --reps 20 --dtype complex64]

prints one JSON line: launches, mean launch time, algorithmic bytes per
launch (input + output elements x element size) and the achieved GB/s.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('kernel', choices=['kraus1q'])
    ap.add_argument('--l', type=int, default=256)
    ap.add_argument('--a', type=int, default=16)
    ap.add_argument('--r', type=int, default=256)
    ap.add_argument('--K', type=int, default=8)
    ap.add_argument('--reps', type=int, default=20)
    ap.add_argument('--dtype', default='complex64')
    a = ap.parse_args()
    print(json.dumps(kraus1q(a.l, a.a, a.r, a.K, a.reps, a.dtype)))


if __name__ == '__main__':
    main()
