"""bench.py's multi-process path on CPU (gloo, world size 2): the rank
bookkeeping, barrier and max-over-ranks timing, and the reference arm, where
rank 0 alone measures and prints while the other rank exits cleanly."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _launch(code_or_args, port, ws=2, timeout=600):
    procs = []
    for r in range(ws):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(ws), MASTER_ADDR='127.0.0.1',
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES='')
        procs.append(subprocess.Popen([sys.executable] + code_or_args, cwd=ROOT, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=timeout)
        except subprocess.TimeoutExpired:
            p.kill()
            raise
        outs.append((p.returncode, out, err))
    return outs


def test_gloo_barrier_and_max_over_ranks():
    code = ("import sys, json; sys.argv = ['bench.py', '--impl', 'reference']; import bench; "
            "args = bench.parse(); rank, ws, local = bench.dist_init(args); "
            "bench.barrier(ws); m = bench.allreduce_max(1.5 + rank, ws); bench.barrier(ws); "
            "print(json.dumps({'rank': rank, 'ws': ws, 'max': m, 'seeds': bench.replica_seeds(rank, 3)}))")
    outs = _launch(['-c', code], _free_port())
    got = [json.loads(o[1].strip().splitlines()[-1]) for o in outs]
    for rc, _, err in outs:
        assert rc == 0, err[-2000:]
    assert sorted(g['rank'] for g in got) == [0, 1]
    assert all(g['ws'] == 2 and g['max'] == 2.5 for g in got)
    seeds = [s for g in got for s in g['seeds']]
    assert len(set(seeds)) == len(seeds) == 6           # replicas evolve disjoint circuits


@pytest.mark.timeout(900)
def test_reference_arm_rank0_only():
    args = ['bench.py', '--impl', 'reference', '--gpus', '2', '--n', '6', '--depth', '2', '--chi', '4', '--kappa',
            '2', '--steps', '1', '--warmup', '1', '--batch', '2']
    outs = _launch(args, _free_port())
    for rc, _, err in outs:
        assert rc == 0, err[-2000:]
    lines = [[ln for ln in o[1].splitlines() if ln.startswith('{')] for o in outs]
    assert len(lines[0]) == 1 and lines[1] == []
    d = json.loads(lines[0][0])
    assert d['impl'] == 'reference' and d['value'] > 0 and d['unit'] == 'gates/s'
    assert d['cpu_baseline']['value'] == d['value'] and d['e2e']['h2d_bytes_per_step'] == 0


def test_uneven_batch_cost_balanced_split():
    # each rank takes its longest-processing-time share of the 256 uneven
    # circuits (reference-trace flops); the shares are disjoint, cover every
    # seed, are even to 1 % in estimated work, and sum/max over ranks agree
    code = ("import sys, json; sys.argv = ['bench.py', '--workload', 'uneven']; import bench; "
            "args = bench.parse(); rank, ws, local = bench.dist_init(args); "
            "seeds, flops, imb = bench.uneven_circuits(rank, ws, 256); "
            "tot = bench.allreduce_sum(len(seeds), ws); m = bench.allreduce_max(10.0 * (rank + 1), ws); "
            "print(json.dumps({'rank': rank, 'seeds': seeds, 'flops': flops, 'imb': imb, 'tot': tot, 'max': m}))")
    outs = _launch(['-c', code], _free_port())
    for rc, _, err in outs:
        assert rc == 0, err[-2000:]
    got = [json.loads(o[1].strip().splitlines()[-1]) for o in outs]
    seeds = [s for g in got for s in g['seeds']]
    assert sorted(seeds) == list(range(256))
    assert all(g['tot'] == 256 and g['max'] == 20.0 for g in got)
    assert got[0]['flops'] == got[1]['flops'] and got[0]['imb'] < 1.01
    # an equal split of the seed range is less even
    from mpdo_gb300.schedule import imbalance, reference_flops
    from mpdo_gb300.workloads import uneven_batch_circuit
    costs = [reference_flops(uneven_batch_circuit(s))[0] for s in range(256)]
    assert imbalance([list(range(128)), list(range(128, 256))], costs) > got[0]['imb']


def test_partition_rule():
    from mpdo_gb300.schedule import imbalance, partition
    costs = [7.0, 5.0, 4.0, 3.0, 3.0, 2.0]
    parts = partition(costs, 2)
    assert parts == [[0, 3, 5], [1, 2, 4]] and imbalance(parts, costs) == 1.0
    assert partition([], 3) == [[], [], []] and partition([1.0], 1) == [[0]]
    with pytest.raises(ValueError):
        partition(costs, 0)


_FIT_CODE = r'''
import json, os, sys
import torch
import torch.distributed as dist
ROOT = os.getcwd()
sys.path[:0] = [ROOT, os.path.join(ROOT, 'tomography-assisted-mpdo-qcircuit_gb300'), os.path.join(ROOT, 'tests')]
from test_multirank_cpu import fit_problem
dist.init_process_group('gloo')
rank, ws = dist.get_rank(), dist.get_world_size()
hist = fit_problem(rank, ws, dist.group.WORLD)
print(json.dumps({'rank': rank, 'loss': hist['loss'], 'W': torch.view_as_real(hist['W']).flatten().tolist()}))
'''


def fit_problem(rank, ws, group):
    """Two Adam steps of the channel fit on four n=4 circuits, this rank's
    share of them (i % ws == rank), marginals from the oracle (differentiable
    in the channel tensor); the gradient and loss summed over ``group``."""
    import torch
    from oracle import channel_fit as C, mpdo_oracle as O
    from mpdo_gb300 import channel_fit as F
    circs = [C.random_circuit(4, 3, s) for s in range(4)]
    data = torch.stack([C.marginals(a, C.kraus(C.hidden_isometry(7, 0.05)), 16, 4) for a in circs])
    mine = [i for i in range(len(circs)) if i % ws == rank]

    class OracleFitter:
        def marginals(self, t):
            out = []
            for i in mine:
                st = O.product_state([[1, 0]] * 4, connected=True)
                O.evolve(st, C.circuit_ops(circs[i], t), chi=16, kappa=4, noisy=True)
                out.append(torch.stack([O.expect_ops(st, {q: C._Z}) for q in range(4)]))
            return torch.stack(out)
    return F.fit(OracleFitter(), data[mine], steps=2, group=group)


@pytest.mark.timeout(900)
def test_channel_fit_gradient_allreduce():
    # config 4 over two ranks: each evolves half of the circuits, the 16 x 4
    # complex gradient is summed once per Adam step, and both ranks end on
    # the W that one process fitting all circuits reaches
    import torch
    outs = _launch(['-c', _FIT_CODE], _free_port())
    for rc, _, err in outs:
        assert rc == 0, err[-2000:]
    got = [json.loads(o[1].strip().splitlines()[-1]) for o in outs]
    ref = fit_problem(0, 1, None)
    w_ref = torch.view_as_real(ref['W']).flatten()
    for g in got:
        assert max(abs(a - b) for a, b in zip(g['loss'], ref['loss'])) < 1e-12 * max(ref['loss'])
        # Adam's early steps are about lr * g / |g| per entry, so entries whose
        # gradient is near zero turn the summation order's rounding into
        # differences far above 1e-16; 1e-6 is 1/20000 of one step (lr 0.02)
        assert (torch.tensor(g['W']) - w_ref).abs().max() < 1e-6
