"""Generate tests/golden/noise.json: the reference's own NoiseChannel
tensors (NoiseChannel.py:20-170; ChipInfo.py presets) in complex128 -- the
chip channels of every preset and the channel constructors at explicit
parameters.

The reference is imported as make_golden.py does it.

Usage (CPU, needs the reference checkout):
    python tests/golden/make_noise_golden.py [--reference PATH]
"""
import argparse
import json
import os

import torch

from make_golden import HERE, _install
from make_tools_golden import _c

CHIPS = ('best', 'medium', 'worst')
ATTRS = ('decayTensor', 'dephasingTensor', 'dpCTensor', 'dpCTensor2', 'apdeCTensor')


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('MPDO_REFERENCE'), required='MPDO_REFERENCE' not in os.environ,
                    help='root of the reference checkout (or set MPDO_REFERENCE)')
    args = ap.parse_args()
    _install(args.reference)
    from MPDOSimulator.NoiseChannel import NoiseChannel
    c128 = torch.complex128
    out = {'generator': 'tests/golden/make_noise_golden.py (reference MPDOSimulator/NoiseChannel.py on CPU)'}
    for chip in CHIPS:
        nc = NoiseChannel(chip=chip, dtype=c128, device='cpu')
        out[chip] = {a: _c(getattr(nc, a)) for a in ATTRS}
    nc = NoiseChannel(dtype=c128, device='cpu')
    out['explicit'] = {
        'depolarization_1': _c(nc.depolarization_noise_channel(p=0.07)),
        'depolarization_2': _c(nc.depolarization_noise_channel(p=0.07, qn=2)),
        'amp_phase_damping': _c(nc.amp_phase_damping_error(time=10.0, T1=50.0, T2=30.0)),
        'decay': _c(nc.decay(0.3, 2.0)),
        'dephasing': _c(nc.dephasing(0.2, 3.0)),
    }
    path = os.path.join(HERE, 'noise.json')
    with open(path, 'w') as f:
        json.dump(out, f)
    print('wrote', os.path.relpath(path))


if __name__ == '__main__':
    main()
