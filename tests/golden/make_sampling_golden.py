"""Generate tests/golden/sampling.json: the reference's own conditional
probabilities p(1 | measured prefix) (Circuit.py:297-332), as its sampler
uses them, on evolved golden circuits, in the Z basis and in a mixed X / Y /
Z orientation (Circuit.py:413-418), for every prefix of length 0..2.

The reference is imported as make_golden.py does it.  Sampling itself is
random; these are the deterministic quantities that drive it.

Usage (CPU, needs the reference checkout):
    python tests/golden/make_sampling_golden.py [--reference PATH]
"""
import argparse
import itertools
import json
import os
import tempfile

import torch

from make_golden import HERE, _install

CIRCUITS = ('noisy_chi_c128', 'unified_chip_c128', 'ideal_chi_c128')


def orientations(n):
    return {'z': [2] * n, 'mixed': [(0, 1, 2)[q % 3] for q in range(n)]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('MPDO_REFERENCE'), required='MPDO_REFERENCE' not in os.environ,
                    help='root of the reference checkout (or set MPDO_REFERENCE)')
    args = ap.parse_args()
    _install(args.reference)
    import MPDOSimulator as S
    from cases import CASES, evolve_case
    torch.manual_seed(0)
    out = {'generator': 'tests/golden/make_sampling_golden.py (reference MPDOSimulator on CPU)'}
    for name in CIRCUITS:
        fn, dtype = CASES[name]
        with tempfile.TemporaryDirectory() as wd:
            c = evolve_case(S, fn(S, dtype, 'cpu', wd), dtype)
        for oname, orient in orientations(c.qnumber).items():
            # one shot sets up the sampler's doubled network (Circuit.py:411-421)
            c.sample(shots=1, orientation=orient, _tqdm_disable=True, _require_counts=False)
            p1 = {}
            for L in range(3):
                for bits in itertools.product((0, 1), repeat=L):
                    p1[''.join(map(str, bits))] = float(c._conditional_prb(list(bits)))
            out[f'{name}:{oname}'] = {'orientation': orient, 'p1': p1}
    path = os.path.join(HERE, 'sampling.json')
    with open(path, 'w') as f:
        json.dump(out, f, indent=1)
    print('wrote', os.path.relpath(path), len(out) - 1, 'tables')


if __name__ == '__main__':
    main()
