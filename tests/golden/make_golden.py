"""Generate the golden fixtures in this directory by running the reference's
own MPDOSimulator (Circuit.py, TNNOptimizer.py, dmOperations.py and the
vendored backend decompositions.py) on the circuits of ``cases.py``.

The reference needs ``tensornetwork`` (pinned 0.4.6, not installed here) and
imports ``matplotlib`` at module load (Tools.py:12-13, absent here).  The
first is replaced by the stand-in under ``_tn_standin/`` (the package's graph
semantics; SVD/QR come from the reference's decompositions.py); the second
by an empty module, as nothing on the evolution path plots.

For every case the fixture holds: the sequence of gate tensors the reference
applied (captured when its gate nodes are created; Circuit.py:102 and
158-166), the truncation markers, the final density matrix (cal_dm), the leg
dimensions of the final state, dmOperations.pauli_expect values on the
final state (dmOperations.py:174-201), and how many SVDs took the
randomized branch of decompositions.py:112-115.

Usage (CPU, needs the reference checkout):
    python tests/golden/make_golden.py [--reference PATH]
"""
import argparse
import json
import os
import sys
import tempfile
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def _install(reference: str):
    sys.path.insert(0, os.path.join(HERE, '_tn_standin'))
    sys.path.insert(0, reference)
    sys.path.insert(0, HERE)
    mpl = types.ModuleType('matplotlib')
    mpl.rcParams = {}                     # Tools.py:22 sets a font
    mpl.pyplot = types.ModuleType('matplotlib.pyplot')
    sys.modules.setdefault('matplotlib', mpl)
    sys.modules.setdefault('matplotlib.pyplot', mpl.pyplot)
    import tensornetwork as tn
    import decompositions as D
    tn.set_backend_module(D)
    return tn, D


def _capture_ops(c, gate_nodes):
    """Pair the circuit's layers with the gate nodes created during evolve."""
    ops, k = [], 0
    for layer, oqs in zip(c.layers, c._oqs_list):
        name = layer.name.lower()
        if 'truncate' in name:
            ops.append({'kind': 'truncate'})
            continue
        if 'barrier' in name or layer.name == 'MeasureZ':
            continue
        n_nodes = len(oqs) if layer.single else 1
        for _ in range(n_nodes):
            axes, t = gate_nodes[k]
            k += 1
            if layer.single:
                q = int(axes[0].split('_')[1])
                ops.append({'kind': '1q', 'q': [q], 'tensor': t})
            else:
                q0, q1 = int(axes[0].split('_')[1]), int(axes[1].split('_')[1])
                ops.append({'kind': '2q', 'q': [q0, q1], 'tensor': t})
    if k != len(gate_nodes):
        raise RuntimeError(f'captured {len(gate_nodes)} gate nodes, paired {k}')
    return ops


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('MPDO_REFERENCE'), required='MPDO_REFERENCE' not in os.environ,
                    help='root of the reference checkout (or set MPDO_REFERENCE)')
    ap.add_argument('--out', default=HERE)
    ap.add_argument('--only', default='', help='comma-separated case names (default: all)')
    args = ap.parse_args()
    tn, D = _install(args.reference)
    counts = {'svd': 0, 'randomized': 0}
    svd0, rsvd0 = D.svd, D._randomized_svd

    def svd(*a, **k):
        counts['svd'] += 1
        return svd0(*a, **k)

    def rsvd(*a, **k):
        counts['randomized'] += 1
        return rsvd0(*a, **k)

    D.svd, D._randomized_svd = svd, rsvd
    gate_nodes = []
    node_init = tn.Node.__init__

    def init(self, tensor, name=None, axis_names=None, backend=None):
        node_init(self, tensor, name=name, axis_names=axis_names, backend=backend)
        if axis_names and any(str(a).startswith('inner_') for a in axis_names):
            gate_nodes.append((list(axis_names), self.tensor.detach().clone()))

    tn.Node.__init__ = init
    import MPDOSimulator as S
    from cases import CASES, HOST_CASES, evolve_case, readout
    torch.manual_seed(0)
    only = set(filter(None, args.only.split(',')))
    for name, (fn, dtype) in {**CASES, **HOST_CASES}.items():
        if only and name not in only:
            continue
        counts.update(svd=0, randomized=0)
        gate_nodes.clear()
        with tempfile.TemporaryDirectory() as wd:
            c = evolve_case(S, fn(S, dtype, 'cpu', wd), dtype)
        out = readout(c, S)
        ops = _capture_ops(c, gate_nodes)
        flat, meta = [], []
        off = 0
        for op in ops:
            m = {'kind': op['kind']}
            if 'tensor' in op:
                t = op['tensor'].to(torch.complex128).numpy()
                m.update(q=op['q'], shape=list(t.shape), offset=off)
                flat.append(t.ravel())
                off += t.size
            meta.append(m)
        info = {'case': name, 'dtype': str(dtype).replace('torch.', ''), 'qn': c.qnumber, 'chi': c.chi,
                'kappa': c.kappa, 'max_truncation_err': c.max_truncation_err, 'ideal': bool(c.ideal),
                'svd_calls': counts['svd'], 'randomized_svd_calls': counts['randomized'], 'dims': out['dims'],
                'ops': meta, 'generator': 'tests/golden/make_golden.py (reference MPDOSimulator on CPU)'}
        path = os.path.join(args.out, f'{name}.npz')
        np.savez_compressed(path, info=np.array(json.dumps(info)), dm=out['dm'].astype(np.complex128),
                            tensors=np.concatenate(flat) if flat else np.zeros(0, np.complex128),
                            pauli=out['pauli'])
        print(f'{name}: n={c.qnumber} svd={counts["svd"]} randomized={counts["randomized"]} '
              f'ops={len(meta)} trace={np.trace(out["dm"]).real:.6f} -> {os.path.relpath(path)}')


if __name__ == '__main__':
    main()
