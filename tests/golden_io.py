"""Reader for the golden fixtures in tests/golden/ (produced by
tests/golden/make_golden.py from the reference's own MPDOSimulator)."""
import glob
import json
import os

import numpy as np
import torch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, '*.npz')))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + '.npz'))
    info = json.loads(str(z['info']))
    flat = z['tensors']
    ops = []
    for m in info['ops']:
        if m['kind'] == 'truncate':
            ops.append(('truncate',))
            continue
        n = int(np.prod(m['shape']))
        t = torch.from_numpy(flat[m['offset']:m['offset'] + n].reshape(m['shape']).copy())
        if m['kind'] == '1q':
            ops.append(('1q', m['q'][0], t))
        else:
            ops.append(('2q', m['q'][0], m['q'][1], t))
    return info, ops, z['dm']


def pauli_values(name):
    """dmOperations.pauli_expect of the reference's final state for the terms
    of cases.PAULI_TERMS."""
    return np.load(os.path.join(GOLDEN, name + '.npz'))['pauli']


def dtype_of(info):
    return torch.complex64 if info['dtype'] == 'complex64' else torch.complex128


def expected_dims(info, k):
    """(left bond, Kraus, right bond) of site k in the reference's final state."""
    d = info['dims'][k]
    return d.get(f'bond_{k - 1}_{k}', 1), d.get(f'I_{k}', 1), d.get(f'bond_{k}_{k + 1}', 1)
