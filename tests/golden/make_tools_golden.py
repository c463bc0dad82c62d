"""Generate tests/golden/tools.json by running the reference's own host
utilities (MPDOSimulator/Tools.py: density2prob, tc_expect, sqrt_matrix,
cal_fidelity, name2matrix, gates_list, count_item, ket_*) on seeded inputs.

The reference's Tools module is imported as make_golden.py does it (the
``tensornetwork`` stand-in under ``_tn_standin/`` and an empty matplotlib).

Usage (CPU, needs the reference checkout):
    python tests/golden/make_tools_golden.py [--reference PATH]
"""
import argparse
import json
import os

import numpy as np
import torch

from make_golden import HERE, _install


def _c(t):
    """complex tensor -> [[re...], [im...]] (nested lists, JSON-able)."""
    a = np.asarray(t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else t, dtype=np.complex128)
    return {'re': a.real.tolist(), 'im': a.imag.tolist(), 'shape': list(a.shape)}


def inputs():
    """The seeded inputs (also rebuilt by the test from the same seed)."""
    g = torch.Generator().manual_seed(11)

    def dm(n):
        a = torch.complex(torch.randn(2 ** n, 2 ** n, dtype=torch.float64, generator=g),
                          torch.randn(2 ** n, 2 ** n, dtype=torch.float64, generator=g))
        r = a @ a.conj().T
        return r / torch.trace(r).real

    rho, sigma = dm(3), dm(3)
    psi = torch.complex(torch.randn(8, dtype=torch.float64, generator=g), torch.randn(8, dtype=torch.float64, generator=g))
    psi = psi / torch.linalg.norm(psi)
    # a pure state (rank one) exercises the eigenvalue clipping of sqrt_matrix
    pure = torch.outer(psi, psi.conj())
    h = torch.tensor([[1, 1], [1, -1]], dtype=torch.complex128) / np.sqrt(2)
    hhh = torch.kron(torch.kron(h, h), h)
    bases = {'Bases': [hhh[:, i].reshape(8, 1) for i in range(8)], 'BasesName': [f'h{i}' for i in range(8)]}
    return dict(rho=rho, sigma=sigma, psi=psi, pure=pure, bases=bases)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('MPDO_REFERENCE'), required='MPDO_REFERENCE' not in os.environ,
                    help='root of the reference checkout (or set MPDO_REFERENCE)')
    args = ap.parse_args()
    _install(args.reference)
    from MPDOSimulator import Tools as T
    x = inputs()
    rho, sigma, psi, pure, bases = x['rho'], x['sigma'], x['psi'], x['pure'], x['bases']
    c128 = torch.complex128
    Z = T.name2matrix('ZII', dtype=c128)
    X = T.name2matrix('IXI', dtype=c128)
    out = {
        'density2prob': T.density2prob(rho),
        'density2prob_tol': T.density2prob(rho, tol=0.1),
        'density2prob_array': np.asarray(T.density2prob(rho, _dict=False)).tolist(),
        'density2prob_bases': T.density2prob(rho, bases=bases),
        'tc_expect_dm': _c(T.tc_expect(Z, rho)),
        'tc_expect_ket': _c(T.tc_expect(X, psi)),
        'tc_expect_list': _c(T.tc_expect([Z, X], rho)),
        'sqrt_matrix': _c(T.sqrt_matrix(rho)),
        'sqrt_matrix_pure': _c(T.sqrt_matrix(pure)),
        'cal_fidelity': float(T.cal_fidelity(rho, sigma).real),
        'cal_fidelity_self': float(T.cal_fidelity(rho, rho).real),
        'cal_fidelity_pure': float(T.cal_fidelity(pure, rho).real),
        'name2matrix_XYZ': _c(T.name2matrix('XYZ', dtype=c128)),
        'gates_list_2': T.gates_list(2),
        'gates_list_xz': T.gates_list(2, ['X', 'Z']),
        'count_item_lists': [[list(k), v] for k, v in T.count_item([[0, 1], [1, 0], [0, 1], [1, 1]]).items()],
        'count_item_strings': [[k, v] for k, v in T.count_item(['011', '100', '011', '001']).items()],
        'count_item_bools': [[list(map(bool, k)), v]
                             for k, v in T.count_item([[True, False], [False, False], [True, False]]).items()],
        'ket_plus': _c(T.ket_plus(c128)), 'ket_minus': _c(T.ket_minus(c128)),
        'ket_hadamard': _c(T.ket_hadamard(c128)), 'ket1': _c(T.ket1(c128)),
        'generator': 'tests/golden/make_tools_golden.py (reference MPDOSimulator/Tools.py on CPU)',
    }
    path = os.path.join(HERE, 'tools.json')
    with open(path, 'w') as f:
        json.dump(out, f, indent=1)
    print('wrote', os.path.relpath(path), f"fidelity={out['cal_fidelity']:.12f}")


if __name__ == '__main__':
    main()
