"""Autotuning of the engine's performance options, with an on-disk cache.

Only options that change nothing beyond rounding are tuned:

* ``tsqr_ratio``  TSQR chunk rows per column (tree depth against chunk size);
* ``bjacobi_bs``  block width of the wide-bond block Jacobi (CTAs per round
                  against work per CTA; 0 = the built-in rule);
* ``bjacobi_fused`` the wide-bond block Jacobi as one thread-block-cluster
                  launch (1) or one launch per tournament round (0); both
                  give the same columns.

A workload class is (device name, precision, chi, kappa).  ``tune`` times a
prefix of a representative circuit of the class (the n-qubit U3 + CZ/CNOT
brickwork with the benchmark noise, enough layers for the bonds to reach
chi) for each candidate value, one option at a time (coordinate descent,
starting from the defaults), and stores the fastest setting in the cache
file (JSON; ``MPDO_GB300_TUNE_CACHE`` or ~/.cache/mpdo_gb300/tune.json).
``options_for`` returns the cached setting (or {}), ``apply`` sets it on an
``Engine`` or ``Batch``.
"""
from __future__ import annotations

import json
import os
import statistics
import time
from typing import Callable, Dict, Optional, Sequence

DEFAULTS = {'tsqr_ratio': 3.0, 'bjacobi_bs': 0, 'bjacobi_fused': 1}
CANDIDATES = {'tsqr_ratio': [2.0, 3.0, 4.0], 'bjacobi_bs': [0, 8, 12, 16, 24, 32], 'bjacobi_fused': [1, 0]}


def cache_path() -> str:
    return os.environ.get('MPDO_GB300_TUNE_CACHE',
                          os.path.join(os.path.expanduser('~'), '.cache', 'mpdo_gb300', 'tune.json'))


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, data: dict) -> None:
    os.makedirs(os.path.dirname(path) or '.', exist_ok=True)
    tmp = path + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def key(device_name: str, dtype: str, chi: int, kappa: int) -> str:
    return f'{device_name}|{dtype}|chi={int(chi)}|kappa={int(kappa)}'


def device_name(device: int = 0) -> str:
    import torch
    return torch.cuda.get_device_name(device) if torch.cuda.is_available() else 'cpu'


def options_for(chi: int, kappa: int, dtype: str = 'complex64', device: int = 0,
                path: Optional[str] = None) -> Dict[str, float]:
    """The cached options of the class, or {} when it was never tuned."""
    ent = _load(path or cache_path()).get(key(device_name(device), dtype, chi, kappa))
    return dict(ent['options']) if ent else {}


def apply(target, options: Dict[str, float]) -> None:
    """Set ``options`` on an Engine or a Batch (every worker engine)."""
    for k, v in options.items():
        target.set_option(k, float(v))


def search(measure: Callable[[Dict[str, float]], float], candidates: Optional[Dict[str, Sequence]] = None,
           start: Optional[Dict[str, float]] = None) -> tuple:
    """Coordinate descent: for each option in turn, the candidate value with
    the smallest ``measure(options)`` (others held at their best so far).
    Returns (best options, best time, every (options, time) measured)."""
    cand = candidates or CANDIDATES
    best = dict(start or DEFAULTS)
    seen = {}

    def timed(opts):
        k = tuple(sorted(opts.items()))
        if k not in seen:
            seen[k] = float(measure(dict(opts)))
        return seen[k]
    best_t = timed(best)
    for name, values in cand.items():
        for v in values:
            trial = dict(best)
            trial[name] = v
            t = timed(trial)
            if t < best_t:
                best, best_t = trial, t
    return best, best_t, [(dict(k), t) for k, t in seen.items()]


def tune(chi: int, kappa: int, dtype: str = 'complex64', device: int = 0, n: int = 24, layers: int = 6,
         repeats: int = 2, path: Optional[str] = None, candidates: Optional[Dict[str, Sequence]] = None) -> dict:
    """Time the candidates on the first ``layers`` layers of the n-qubit
    benchmark-style circuit of this class, store and return the fastest
    setting: dict(options, seconds, default_seconds, trials)."""
    import torch
    from .engine import Chain, Engine
    from .workloads import build_circuit, u3_brickwork
    w = u3_brickwork(n=n, depth=layers, chi=chi, kappa=kappa, seed=0)
    c = build_circuit(w, dtype=torch.complex64 if dtype == 'complex64' else torch.complex128,
                      device=f'cuda:{device}')
    ops = c._engine_ops()
    eng = Engine(device)

    def run():
        ch = Chain([[1, 0]] * w.n, dtype=dtype, connected=True, engine=eng)
        for op in ops:
            if op[0] == '1q':
                ch.apply_1q(op[1], op[2])
            elif op[0] == '2q':
                ch.apply_2q(op[1], op[2], 2.718281828459045e-8)
            elif op[0] == 'truncate':
                ch.truncate(w.chi, w.kappa, None, True)
            else:
                ch.kappa_truncate(w.kappa, None)
        eng.sync()
        del ch

    def measure(opts):
        apply(eng, opts)
        run()                                   # warm-up at these options
        ts = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            run()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts)
    best, best_t, trials = search(measure, candidates)
    default_t = next(t for o, t in trials if o == DEFAULTS)
    p = path or cache_path()
    data = _load(p)
    ent = {'options': best, 'seconds': best_t, 'default_seconds': default_t,
           'workload': f'{w.name}, first {layers} layers', 'trials': trials}
    data[key(device_name(device), dtype, chi, kappa)] = ent
    _store(p, data)
    return ent
