"""The autotuner's search and cache (mpdo_gb300.autotune), on the CPU with a
stand-in timing function; the GPU run that fills the cache is in
test_autotune_gpu below."""
import json

import pytest
import torch


def test_coordinate_descent_and_cache(tmp_path, monkeypatch):
    from mpdo_gb300 import autotune as A
    cost = {('tsqr_ratio', 2.0): 3.0, ('tsqr_ratio', 3.0): 2.0, ('tsqr_ratio', 4.0): 2.5,
            ('bjacobi_bs', 0): 1.0, ('bjacobi_bs', 8): 0.5, ('bjacobi_bs', 12): 0.7, ('bjacobi_bs', 16): 0.9,
            ('bjacobi_bs', 24): 1.2, ('bjacobi_bs', 32): 1.4, ('bjacobi_fused', 1): 0.0, ('bjacobi_fused', 0): 0.3}
    calls = []

    def measure(o):
        calls.append(dict(o))
        return (cost[('tsqr_ratio', o['tsqr_ratio'])] + cost[('bjacobi_bs', o['bjacobi_bs'])]
                + cost[('bjacobi_fused', o['bjacobi_fused'])])
    best, t, trials = A.search(measure)
    assert best == {'tsqr_ratio': 3.0, 'bjacobi_bs': 8, 'bjacobi_fused': 1} and t == 2.5
    assert len(calls) == len({tuple(sorted(c.items())) for c in calls})      # no setting timed twice
    path = str(tmp_path / 'tune.json')
    monkeypatch.setenv('MPDO_GB300_TUNE_CACHE', path)
    assert A.options_for(64, 4) == {}
    data = {A.key(A.device_name(0), 'complex64', 64, 4): {'options': best, 'seconds': t}}
    with open(path, 'w') as f:
        json.dump(data, f)
    assert A.options_for(64, 4) == best and A.options_for(128, 4) == {}

    class Target:
        def __init__(self):
            self.set = {}

        def set_option(self, k, v):
            self.set[k] = v
    tg = Target()
    A.apply(tg, best)
    assert tg.set == {'tsqr_ratio': 3.0, 'bjacobi_bs': 8.0, 'bjacobi_fused': 1.0}


@pytest.mark.gpu
def test_autotune_gpu(tmp_path):
    mg = pytest.importorskip('mpdo_gb300')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    mg.build()
    from mpdo_gb300 import autotune as A
    path = str(tmp_path / 'tune.json')
    ent = A.tune(16, 2, n=12, layers=4, repeats=1, path=path,
                 candidates={'tsqr_ratio': [2.0, 3.0], 'bjacobi_bs': [0, 8]})
    assert ent['seconds'] <= ent['default_seconds']
    assert set(ent['options']) == {'tsqr_ratio', 'bjacobi_bs', 'bjacobi_fused'}
    assert A.options_for(16, 2, path=path) == ent['options']
