"""Generate tests/golden/dmops.json: the reference's own dmOperations
readouts (trace_rho, trace_rho2, trace_rho_rho, trace_composited_rho,
trace_composited_rho2; dmOperations.py:18-132) on two evolved golden
circuits of four qubits, on the full doubled networks and with qubits 1 and
3 traced out (reduce_dmNodes, dmOperations.py:18-37).

The reference is imported as make_golden.py does it.

Usage (CPU, needs the reference checkout):
    python tests/golden/make_dmops_golden.py [--reference PATH]
"""
import argparse
import json
import os
import tempfile

import torch

from make_golden import HERE, _install

PAIR = ('noisy_err_c128', 'unified_chip_c128')
TRACED = [1, 3]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('MPDO_REFERENCE'), required='MPDO_REFERENCE' not in os.environ,
                    help='root of the reference checkout (or set MPDO_REFERENCE)')
    args = ap.parse_args()
    _install(args.reference)
    import MPDOSimulator as S
    from MPDOSimulator import dmOperations as D
    from cases import CASES, evolve_case
    torch.manual_seed(0)
    circuits = []
    for name in PAIR:
        fn, dtype = CASES[name]
        with tempfile.TemporaryDirectory() as wd:
            circuits.append(evolve_case(S, fn(S, dtype, 'cpu', wd), dtype))
    n = circuits[0].qnumber

    def nodes(c, traced):
        d = c.cal_dmNodes()
        if traced:
            D.reduce_dmNodes(d[:n], d[n:], reduced_index=traced)
        return d

    out = {'generator': 'tests/golden/make_dmops_golden.py (reference MPDOSimulator/dmOperations.py on CPU)',
           'pair': list(PAIR), 'traced': TRACED}
    for tag, traced in (('full', []), ('reduced', TRACED)):
        a, b = nodes(circuits[0], traced), nodes(circuits[1], traced)
        out[tag] = {
            'trace_rho': float(D.trace_rho(a)),
            'trace_rho2': float(D.trace_rho2(a)),
            'trace_rho_rho': float(D.trace_rho_rho(a, b)),
            'trace_composited_rho': float(D.trace_composited_rho(a, b)),
            'trace_composited_rho2': float(D.trace_composited_rho2(a, b)),
        }
    path = os.path.join(HERE, 'dmops.json')
    with open(path, 'w') as f:
        json.dump(out, f, indent=1)
    print('wrote', os.path.relpath(path), out['full'], out['reduced'])


if __name__ == '__main__':
    main()
