"""The drop-in NoiseChannel (MPDOSimulator/NoiseChannel.py, ChipInfo.py)
against the reference's own channel tensors (tests/golden/noise.json, made
by tests/golden/make_noise_golden.py): every chip preset's decay, dephasing,
1q / 2q depolarising and amplitude-phase-damping tensors, and the
constructors at explicit parameters, in complex128."""
import json
import os

import numpy as np
import pytest
import torch

import golden_io as G

with open(os.path.join(G.GOLDEN, 'noise.json')) as _f:
    REF = json.load(_f)


def _arr(d):
    return (np.asarray(d['re']) + 1j * np.asarray(d['im'])).reshape(d['shape'])


@pytest.mark.parametrize('chip', ['best', 'medium', 'worst'])
def test_chip_channels_match_reference(chip):
    from MPDOSimulator.NoiseChannel import NoiseChannel
    nc = NoiseChannel(chip=chip, dtype=torch.complex128, device='cpu')
    for attr, ref in REF[chip].items():
        got = getattr(nc, attr).detach().cpu().numpy()
        assert got.shape == tuple(ref['shape']), attr
        np.testing.assert_allclose(got, _arr(ref), rtol=0, atol=1e-14, err_msg=attr)


def test_channel_constructors_match_reference():
    from MPDOSimulator.NoiseChannel import NoiseChannel
    nc = NoiseChannel(dtype=torch.complex128, device='cpu')
    got = {'depolarization_1': nc.depolarization_noise_channel(p=0.07),
           'depolarization_2': nc.depolarization_noise_channel(p=0.07, qn=2),
           'amp_phase_damping': nc.amp_phase_damping_error(time=10.0, T1=50.0, T2=30.0),
           'decay': nc.decay(0.3, 2.0), 'dephasing': nc.dephasing(0.2, 3.0)}
    for k, ref in REF['explicit'].items():
        np.testing.assert_allclose(got[k].detach().cpu().numpy(), _arr(ref), rtol=0, atol=1e-14, err_msg=k)
