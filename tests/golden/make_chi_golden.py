"""Generate tests/golden/chi.json from the reference's own chi-matrix
fixtures (MPDOSimulator/chi/ideal_cz.mat and czDefault.mat, key 'exp',
16 x 16 complex): the matrices and the Kraus tensor the reference's
RealNoise.czExp_channel (RealNoise.py:22-170) makes from each, in complex128.

The reference is imported as make_golden.py does it.

Usage (CPU, needs the reference checkout):
    python tests/golden/make_chi_golden.py [--reference PATH]
"""
import argparse
import json
import os

import numpy as np
import torch

from make_golden import HERE, _install
from make_tools_golden import _c

FILES = ('ideal_cz.mat', 'czDefault.mat')


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('MPDO_REFERENCE'), required='MPDO_REFERENCE' not in os.environ,
                    help='root of the reference checkout (or set MPDO_REFERENCE)')
    args = ap.parse_args()
    _install(args.reference)
    from MPDOSimulator import RealNoise as R
    out = {'generator': 'tests/golden/make_chi_golden.py (reference MPDOSimulator/RealNoise.py on CPU)'}
    for fn in FILES:
        path = os.path.join(args.reference, 'MPDOSimulator', 'chi', fn)
        chi = np.asarray(R.readExpChi(path), dtype=np.complex128)
        kraus = R.czExp_channel(filename=path, dtype=torch.complex128)
        out[fn] = {'chi': _c(chi), 'kraus': _c(kraus)}
    path = os.path.join(HERE, 'chi.json')
    with open(path, 'w') as f:
        json.dump(out, f)
    print('wrote', os.path.relpath(path), {k: v['kraus']['shape'] for k, v in out.items() if k != 'generator'})


if __name__ == '__main__':
    main()
