"""Golden readouts of the n=32, chi=64, kappa=4 U3 + CZ/CNOT brickwork from the
complex128 oracle (exact SVDs), for the GPU parity tests at the benchmarked
shape.

The circuit is ``mpdo_gb300.workloads.u3_brickwork`` (seeded angles and gate
picks); Kraus tensors come from the oracle's restatement of the reference's
builders (depolarising p1 then amplitude damping gamma after every U3,
2q depolarising p2 after every CZ / CNOT: NoiseChannel.py:51-170,
Circuit.py:88-100, 141-155).  The evolution is ``oracle.engine_path``: the
reference's truncation placement and rules (Circuit.py:469-491,
TNNOptimizer.py:87-197, decompositions.py:108-146) in the engine's order of
operations (pending 2q gates fused into the QR sweep; only the right site of
each pair is decomposed in the SVD sweep, its left neighbour being an
isometry), which ``tests/test_engine_path_oracle.py`` pins against the
reference order.  Every factorisation runs in complex128.

Recorded: Re Tr(rho Z_i), Re Tr(rho Z_i Z_{i+1}), Tr(rho), the 1-qubit
Z-basis marginals and the 2-qubit reduced density matrices of neighbouring
pairs (unnormalised), the per-bond discarded weight of every truncate layer
and the leg dimensions of the final state.

``--max-err`` sets the reference's relative truncation error
(``max_truncation_err``, TNNOptimizer.py:111-134 and 164-197).

``--conditioning K`` also evolves the circuit again under rounding-level
changes -- once with LAPACK's QR-iteration SVD driver (gesvd) in place of
torch's default, and once per seed 1..K with every site multiplied by
(1 + 1e-13 g), g ~ N(0, 1), after the first truncate layer -- and records the
largest change of each readout over these variants: how far the algorithm
itself (complex128 throughout) moves when only its rounding changes.  Without
an error rule the chi cap keeps singular values at the rounding floor
(decompositions.py:121-140 keeps min(chi, rows, cols) values) and the split
puts sqrt(S) on both factors (TNNOptimizer.py:129-134), so rounding noise of
relative size eps enters the sites at sqrt(eps); the kappa pass then selects
Kraus directions by singular values that carry that noise.  No implementation
can agree with another one more closely than this spread.  With an error
rule that drops the rounding floor (``--max-err 1e-6``) the spread falls to
the rounding level.

``--fp32-storage`` records, beside it, how far the same evolution moves when
the state is stored in complex64 (every factorisation still in complex128,
as the oracle does for complex64 inputs): the floor that rounding the
state to single precision after every operation sets for any complex64
implementation.

    python tests/golden/make_bench_parity.py --depth 20 --conditioning 2 --out tests/golden/bench_n32_d20.json
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, 'tomography-assisted-mpdo-qcircuit_gb300')):
    if p not in sys.path:
        sys.path.insert(0, p)

import torch  # noqa: E402

from oracle import mpdo_oracle as O, engine_path as EP  # noqa: E402
from mpdo_gb300.workloads import u3_brickwork  # noqa: E402

Z = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex128)


def oracle_ops(w):
    dec = O.amplitude_damping(w.noise['gamma'])
    dep = O.depolarization(w.noise['p1'])
    dp2 = O.depolarization(w.noise['p2'], 2)
    ops = []
    for L in w.layers:
        if L[0] == '1q':
            ops.append(('1q', L[3], O.noisy_1q(dec, dep, O.gate_1q(L[1], *L[2]))))
        elif L[0] == '2q':
            ops.append(('2q', L[3], L[4], O.noisy_2q(dp2, O.gate_2q(L[1], *L[2]))))
        else:
            ops.append(('truncate',))
    return ops


def readouts(st):
    n = st.n
    out = {'trace': float(O.trace(st))}
    out['z'] = [float(O.expect_ops(st, {q: Z})) for q in range(n)]
    out['zz'] = [float(O.expect_ops(st, {q: Z, q + 1: Z})) for q in range(n - 1)]
    marg = []
    for q in range(n):
        r = O.reduced_dm(st, [q]).numpy()
        marg.append([float(r[0, 0].real), float(r[1, 1].real)])
    out['marginals'] = marg
    rdm2 = []
    for q in range(n - 1):
        r = O.reduced_dm(st, [q, q + 1]).numpy()
        rdm2.append([[float(x.real), float(x.imag)] for x in r.ravel()])
    out['rdm2'] = rdm2
    return out


def diff(x, y):
    """Largest change of each readout between two results."""
    return {'z': max(abs(p - q) for p, q in zip(x['z'], y['z'])),
            'zz': max(abs(p - q) for p, q in zip(x['zz'], y['zz'])),
            'trace': abs(x['trace'] - y['trace']),
            'marginals': max(abs(p[k] - q[k]) for p, q in zip(x['marginals'], y['marginals']) for k in (0, 1)),
            'rdm2': max(abs(complex(*u) - complex(*v)) for p, q in zip(x['rdm2'], y['rdm2']) for u, v in zip(p, q))}


def _svd_gesvd(M):
    import scipy.linalg
    u, s, vh = scipy.linalg.svd(M.numpy(), full_matrices=False, lapack_driver='gesvd')
    return torch.from_numpy(u), torch.from_numpy(s), torch.from_numpy(vh)


def evolve(w, ops, max_err, perturb=0.0, pseed=1, driver=None, log=True, dtype=torch.complex128):
    """engine_path's evolution, recording every SVD-sweep step's discarded
    weight sum(s_rest^2) / sum(s^2) (bonds n-2 .. 0 run right to left)."""
    disc_steps, discarded = [], []
    orig_trunc, orig_svd = O.svd_truncate, O._svd128

    def rec(M, max_sv=None, max_e=None, relative=False, randomized=False):
        u, s, vh, rest = orig_trunc(M, max_sv, max_e, relative, randomized)
        tot = float((s ** 2).sum() + (rest ** 2).sum())
        disc_steps.append(float((rest ** 2).sum()) / tot if tot > 0 else 0.0)
        return u, s, vh, rest
    O.svd_truncate = rec
    if driver == 'gesvd':
        O._svd128 = _svd_gesvd
    gen = torch.Generator().manual_seed(pseed)
    st = O.product_state([[1, 0]] * w.n, connected=True, dtype=dtype)
    ch = EP.EngineChain(st)
    if dtype != torch.complex128:
        ops = [(o[0],) + tuple(x.to(dtype) if torch.is_tensor(x) else x for x in o[1:]) for o in ops]
    t0, li = time.time(), 0
    try:
        for op in ops:
            if op[0] == '1q':
                ch.apply_1q(op[1], op[2])
            elif op[0] == '2q':
                i, t = O.orient_2q(op[1], op[2], op[3])
                ch.apply_2q(i, t)
            elif O.connected(st):
                # EngineChain.truncate with the SVD sweep's steps recorded
                disc_steps.clear()
                ch._qr_sweep()
                ch._svd_sweep(w.chi, max_err)
                discarded.append(list(reversed(disc_steps)))
                ch.materialize_all()
                O.svd_kappa(st, w.kappa, max_err)
                li += 1
                if perturb and li == 1:
                    st.sites = [x * (1 + perturb * torch.randn(x.shape, generator=gen, dtype=torch.float64))
                                for x in st.sites]
                if log and li % 10 == 0:
                    print(f'  truncate layer {li}  {time.time() - t0:.0f} s', flush=True)
        ch.materialize_all()
    finally:
        O.svd_truncate, O._svd128 = orig_trunc, orig_svd
    st.sites = [x.to(torch.complex128) for x in st.sites]
    res = readouts(st)
    res.update({'discarded': discarded, 'dims': [list(s.shape) for s in st.sites]})
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--n', type=int, default=32)
    ap.add_argument('--depth', type=int, default=20)
    ap.add_argument('--chi', type=int, default=64)
    ap.add_argument('--kappa', type=int, default=4)
    ap.add_argument('--seed', type=int, default=0)
    ap.add_argument('--max-err', type=float, default=None)
    ap.add_argument('--conditioning', type=int, default=0, help='perturbation seeds (plus one gesvd run)')
    ap.add_argument('--fp32-storage', action='store_true')
    ap.add_argument('--threads', type=int, default=0)
    ap.add_argument('--out', required=True)
    a = ap.parse_args()
    if a.threads:
        torch.set_num_threads(a.threads)
    w = u3_brickwork(n=a.n, depth=a.depth, chi=a.chi, kappa=a.kappa, seed=a.seed)
    ops = oracle_ops(w)
    res = evolve(w, ops, a.max_err)
    if a.conditioning:
        variants = [('gesvd', dict(driver='gesvd'))] + [(f'perturbation seed {k}', dict(perturb=1e-13, pseed=k))
                                                         for k in range(1, a.conditioning + 1)]
        cond = {'variants': [v[0] for v in variants],
                'perturbation': 'every site x (1 + 1e-13 g), g ~ N(0, 1), after the first truncate layer'}
        for name, kw in variants:
            d = diff(res, evolve(w, ops, a.max_err, **kw))
            cond[name] = d
            for k, v in d.items():
                cond[k] = max(cond.get(k, 0.0), v)
            print(name, {k: f'{v:.2e}' for k, v in d.items()}, flush=True)
        res['conditioning'] = cond
    if a.fp32_storage:
        d = diff(res, evolve(w, ops, a.max_err, dtype=torch.complex64))
        d['how'] = 'state stored in complex64 after every operation, factorisations in complex128'
        res['fp32_storage'] = d
        print('fp32 storage', {k: (f'{v:.2e}' if isinstance(v, float) else v) for k, v in d.items()}, flush=True)
    res.update({'workload': w.name, 'n': w.n, 'depth': w.depth, 'chi': w.chi, 'kappa': w.kappa, 'seed': a.seed,
                'max_err': a.max_err, 'noise': w.noise,
                'oracle': 'oracle.engine_path, complex128, exact SVDs (LAPACK)', 'torch': torch.__version__})
    with open(a.out, 'w') as f:
        json.dump(res, f)
    print('wrote', a.out, flush=True)


if __name__ == '__main__':
    main()
