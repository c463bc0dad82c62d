#!/usr/bin/env python
"""Benchmark of the MPDO noisy-circuit hot path: gates/s (batched and plain)
and grad-evals/s of the adjoint.

Circuit (the n=32, chi=64, kappa=4 workload): 32 qubits, depth 20 (U3 on every
qubit, then CZ/CNOT brickwork), 1q depolarising 1e-3 + amplitude damping 1e-3
after every 1q gate, 2q depolarising 1e-2 after every 2q gate, a truncate()
after every sublayer, complex64; 950 gates and 40 truncate layers.

One step = one batch of --batch independent circuits of that shape (seeds
0..B-1) through the batched engine (--workers worker engines, each with its
own stream and memory pool).
value:    gates/s over the K timed steps, CUDA events on an idle stream around
          the synchronous batch call (Kraus tensors are host data by design:
          they travel as kernel parameters), L2 flushed between steps.
e2e:      the same circuits through the public API (MPDOSimulator.evolve_batch
          on TensorCircuit objects built per step, host product states in,
          <Z_i>, <Z_i Z_i+1> and per-bond discarded weights out).
plain:    one circuit through one engine and through TensorCircuit.evolve.
parity:   the plain run's readouts against the complex128 oracle's
          (tests/golden/bench_n32_d20.json) beside the spread of complex128
          oracle runs that differ only in rounding (this form of the workload
          is ill-conditioned), and the same circuit with the reference's
          relative truncation error 1e-6 (well conditioned) against its
          oracle fixture and the floor that single-precision storage sets.
grad:     grad-evals/s of the adjoint on the hardware-efficient ansatz (n=24,
          12 layers of RY, RZ and a CZ ladder, chi=32, kappa=4, one
          depolarising probability per gate type, Ising energy), complex64,
          and its cost against its own forward pass.
roofline: the dominant kernel class of one profiled batch (its algorithmic
          flops per launch over its mean launch time) and, per the
          reference's algorithm, the flops of the reference's shape trace of
          the step (its SVDs of contracted pairs, QRs, kappa SVDs) over the
          step time; both against the nominal FP32 SIMT rate (the kernels run
          on the FP32 pipe) and the measured bf16 tensor peak.
cpu_baseline / --impl reference: the CPU oracle (restatement of the
          reference path, torch CPU, with the reference's randomized SVD for
          capped SVDs of >= 1e4 elements) timing layer 1 of the seed-0
          circuit in full (no extrapolation).

Multi-GPU (torchrun, N > 1): independent replicas, each rank its own batch of
seeds; value = total gates / max time over ranks.
"""
import argparse
import json
import os

# one hardware work queue per batch worker stream (must precede CUDA init)
os.environ.setdefault('CUDA_DEVICE_MAX_CONNECTIONS', '32')
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, 'tomography-assisted-mpdo-qcircuit_gb300')
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = 'gates/s & grad-evals/s at n=32 χ=64 κ=4: batched/adjoint vs plain, ≤1e-5 err'
FP32_SIMT_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12    # 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz
GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--n', type=int, default=32)
    ap.add_argument('--depth', type=int, default=20)
    ap.add_argument('--chi', type=int, default=64)
    ap.add_argument('--kappa', type=int, default=4)
    ap.add_argument('--dtype', default='complex64')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--batch', type=int, default=24, help='independent circuits per step (seeds)')
    ap.add_argument('--workers', type=int, default=24, help='worker engines of the batch runner')
    ap.add_argument('--plain-steps', type=int, default=1, help='timed single-circuit runs (reported as plain)')
    ap.add_argument('--plain-warmup', type=int, default=1)
    ap.add_argument('--grad-steps', type=int, default=2, help='timed adjoint gradients (0: none)')
    ap.add_argument('--grad-warmup', type=int, default=1)
    ap.add_argument('--no-parity', action='store_true')
    ap.add_argument('--autotune', action='store_true',
                    help='apply the autotuner\'s cached options for this class (tuning first when none are cached)')
    ap.add_argument('--workload', default='u3_brickwork', choices=['u3_brickwork', 'uneven'],
                    help='uneven: the 256-circuit uneven batch (one step = the whole batch)')
    ap.add_argument('--circuits', type=int, default=256, help='uneven: circuits (seeds 0..K-1) over all ranks')
    ap.add_argument('--sequential', action='store_true',
                    help='uneven: also run every circuit one at a time through the plain path (long)')
    return ap.parse_args()


def dist_init(args):
    import torch
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if ws > 1:
        import torch.distributed as dist
        backend = 'nccl' if torch.cuda.is_available() and args.impl == 'gb300' else 'gloo'
        dist.init_process_group(backend=backend)
    return rank, ws, local


def replica_seeds(rank, per_rank):
    """Circuit seeds of one rank: every rank evolves its own, disjoint set."""
    return [rank * per_rank + k for k in range(per_rank)]


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device='cuda' if dist.get_backend() == 'nccl' else 'cpu')
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------- workload --
def workload(args, seed=0):
    from mpdo_gb300.workloads import u3_brickwork
    return u3_brickwork(n=args.n, depth=args.depth, chi=args.chi, kappa=args.kappa, seed=seed)


def host_ops(w, dtype, device='cuda:0'):
    """The circuit as the drop-in API builds it and the engine operations its
    evolve() performs (Kraus tensors by the API's own builders)."""
    import torch
    from mpdo_gb300.workloads import build_circuit
    c = build_circuit(w, dtype=torch.complex64 if dtype == 'complex64' else torch.complex128, device=device)
    return c, c._engine_ops()


def run_chain(ops, w, dtype, eng, max_err=None, discarded=None):
    from mpdo_gb300 import Chain
    ch = Chain([[1, 0]] * w.n, dtype=dtype, connected=True, engine=eng)
    for op in ops:
        if op[0] == '1q':
            ch.apply_1q(op[1], op[2])
        elif op[0] == '2q':
            ch.apply_2q(op[1], op[2], 2.718281828459045e-8)
        elif op[0] == 'truncate':
            d = ch.truncate(w.chi, w.kappa, max_err, True, report=discarded is not None)
            if discarded is not None:
                discarded.append(d)
        else:
            ch.kappa_truncate(w.kappa, max_err)
    return ch


def program(w, ops, dtype):
    return dict(n=w.n, dtype=dtype, vectors=[[1, 0]] * w.n, connected=True, chi=w.chi, kappa=w.kappa,
                max_err=None, noisy=True, ops=ops, z=True, zz=True, discarded=True)


# ---------------------------------------------- reference shape trace (8d) --
def reference_trace_flops(w, K1=8, K2=16):
    """Flops of the reference's algorithm on this circuit from its shape trace
    (mpdo_gb300.schedule.reference_flops)."""
    from mpdo_gb300.schedule import reference_flops
    return reference_flops(w, K1, K2)


# ----------------------------------------------------------------- clocks --
class ClockSampler:
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.device), f'--query-gpu={self.FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(',')]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            if self.path and os.path.exists(self.path):
                os.remove(self.path)
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['clock sampling unavailable']}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == 'active'})
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows)}


# ------------------------------------------------------------ CPU oracle --
class CpuLayer:
    """The CPU oracle (the reference's algorithm restated in torch) on layer 1
    of the workload, timed in full: layer 0 is evolved once (bonds reach chi)
    and each sample times the whole of layer 1 (its U3 sublayer, 2q sublayer
    and both truncates) on a copy of that state.  Factorisations in
    complex128 with the state stored in complex64 (the Arm hosts' LAPACK
    aborts on some complex64 SVDs); capped SVDs of >= 1e4 elements take the
    reference's randomized branch (decompositions.py:112-115), as its stock
    code path does."""

    def __init__(self, w, threads=None, randomized=True):
        import torch
        from oracle import mpdo_oracle as O
        self.O, self.w, self.randomized = O, w, randomized
        if threads:
            torch.set_num_threads(threads)
        self.threads = torch.get_num_threads()
        dt = torch.complex64
        dec = O.amplitude_damping(w.noise['gamma'], dt)
        dep = O.depolarization(w.noise['p1'], 1, dt)
        dp2 = O.depolarization(w.noise['p2'], 2, dt)
        layers, cur, subs = [], [], 0
        for L in w.layers:
            if L[0] == '1q':
                cur.append(('1q', L[3], O.noisy_1q(dec, dep, O.gate_1q(L[1], *L[2], dtype=dt))))
            elif L[0] == '2q':
                cur.append(('2q', L[3], L[4], O.noisy_2q(dp2, O.gate_2q(L[1], *L[2], dtype=dt))))
            else:
                cur.append(('truncate',))
                subs += 1
                if subs % 2 == 0:
                    layers.append(cur)
                    cur = []
        self.layer1 = layers[1]
        self.gates = sum(1 for op in self.layer1 if op[0] != 'truncate')
        self.state = O.product_state([[1, 0]] * w.n, connected=True, dtype=dt)
        O.evolve(self.state, layers[0], chi=w.chi, kappa=w.kappa, noisy=True, randomized=randomized)

    def sample(self):
        secs, info = self.O.time_layer(self.state.clone(), self.layer1, self.w.chi, self.w.kappa,
                                       budget_s=float('inf'), randomized=self.randomized)
        return self.gates / secs, secs

    def describe(self):
        import torch
        return (f'layer 1 ({self.gates} gates: 32 U3, 16 two-qubit gates, 2 truncates) of the seed-0 circuit on '
                f'the CPU oracle, timed in full, torch {torch.__version__}, {self.threads} threads, SVDs as the '
                f'reference takes them (randomized for capped matrices of >= 1e4 elements, exact otherwise)')


def reference_arm(args):
    rank, ws, _ = dist_init(args)
    if rank != 0:
        return
    w = workload(args)
    cpu = CpuLayer(w, threads=os.cpu_count() or 1)
    vals, secs = [], []
    for k in range(args.warmup + args.steps):
        v, s = cpu.sample()
        if k >= args.warmup:
            vals.append(v)
            secs.append(s)
    val = len(vals) / sum(1.0 / v for v in vals)        # gates per total second
    out = {'metric': METRIC, 'value': val, 'unit': 'gates/s', 'n_gpus': args.gpus, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': 1e3 * statistics.mean(secs), 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic', 'impl': 'reference',
           'config': {'workload': f'{max(1, args.batch)} independent circuits of {w.name}, seeds 0..'
                                  f'{max(1, args.batch) - 1}', 'n': w.n, 'depth': w.depth, 'chi': w.chi,
                      'kappa': w.kappa, 'circuits_per_step': max(1, args.batch),
                      'step': 'circuits run one after another; each step times one steady-state layer of the '
                              'seed-0 circuit in full'},
           'cpu_baseline': {'value': val, 'unit': 'gates/s', 'cores': cpu.threads, 'kind': 'port',
                            'sample': cpu.describe()},
           'e2e': {'value': val, 'unit': 'gates/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------- GPU arm --
def _roofline(prof, peaks):
    """Dominant kernel class of a profiled run: its algorithmic flops (bytes
    for the memory-bound site kernels) per launch over its mean launch time."""
    dom = max(prof, key=lambda k: prof[k]['ms'])
    d = prof[dom]
    bf16 = peaks.get('bf16_tflops')
    if dom in ('kraus1q', 'mix2q', 'other'):
        achieved = d['bytes'] / (d['ms'] / 1e3) / 1e9
        peak = peaks.get('hbm_gbs', 6800.0)
        roof = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                'peak_source': 'measured (MEASURED_PEAKS.json)' if 'hbm_gbs' in peaks else 'fallback'}
        per_launch_alg = d['bytes'] / max(1, d['launches'])
    else:
        achieved = d['flops'] / (d['ms'] / 1e3) / 1e12
        roof = {'bound': 'tensor', 'pipe': 'fp32_simt', 'achieved': achieved, 'peak': FP32_SIMT_NOMINAL_TFLOPS,
                'unit': 'TFLOP/s', 'frac': achieved / FP32_SIMT_NOMINAL_TFLOPS,
                'peak_source': 'nominal FP32 SIMT rate (152 SMs x 128 lanes x 2 flops x 2.07 GHz): the kernels run '
                               'on the FP32 pipe and MEASURED_PEAKS.json holds no FP32 figure',
                'frac_of_measured_bf16_tensor': achieved / bf16 if bf16 else None}
        per_launch_alg = d['flops'] / max(1, d['launches'])
    roof.update({'kernel': dom, 'launches': d['launches'], 'kernel_ms': d['ms'],
                 'mean_launch_us': 1e3 * d['ms'] / max(1, d['launches']),
                 'share_of_kernel_time': d['ms'] / (sum(v['ms'] for v in prof.values()) or 1),
                 'algorithmic_per_launch': per_launch_alg, 'traffic': None})
    tfile = os.path.join(ROOT, 'profiles', 'traffic.json')
    if os.path.exists(tfile):
        tr = json.load(open(tfile)).get(dom)
        if tr:
            roof['traffic'] = tr.get('bytes_per_launch')
    return roof


def _sum_profiles(profs):
    out = {}
    for p in profs:
        for k, v in p.items():
            if k in ('wide_bonds', 'phases'):
                continue
            o = out.setdefault(k, dict(launches=0, ms=0.0, flops=0.0, bytes=0.0))
            for f in o:
                o[f] += v[f]
    return out


def _readouts(ch, n):
    import numpy as np
    Z = np.diag([1, -1]).astype(complex)
    return {'trace': ch.expect_ops({}), 'z': [ch.expect_ops({q: Z}) for q in range(n)],
            'zz': [ch.expect_ops({q: Z, q + 1: Z}) for q in range(n - 1)],
            'marginals': [list(ch.probs([q])) for q in range(n)],
            'rdm2': [ch.reduced_dm([q, q + 1]) for q in range(n - 1)]}


def _errors(got, ref):
    import numpy as np
    r2 = [np.array([complex(*v) for v in m]).reshape(4, 4) for m in ref['rdm2']]
    return {'trace': abs(got['trace'] - ref['trace']),
            'z': float(np.abs(np.array(got['z']) - ref['z']).max()),
            'zz': float(np.abs(np.array(got['zz']) - ref['zz']).max()),
            'marginals': float(np.abs(np.array(got['marginals']) - np.array(ref['marginals'])).max()),
            'rdm2': float(max(np.abs(a - b).max() for a, b in zip(got['rdm2'], r2)))}


def parity(args, w, ops, eng, plain_chain, plain_disc):
    """Errors of the engine against the complex128 oracle fixtures (seed 0,
    n=32, depth 20, chi=64, kappa=4)."""
    import numpy as np
    keys = ('trace', 'z', 'zz', 'marginals', 'rdm2')
    out = {'vs': 'complex128 oracle (oracle/engine_path.py, exact LAPACK SVDs): tests/golden/'}
    f = os.path.join(GOLDEN, 'bench_n32_d20.json')
    if (w.n, w.depth, w.chi, w.kappa) != (32, 20, 64, 4) or not os.path.exists(f):
        out['skipped'] = 'fixtures exist for n=32, depth 20, chi=64, kappa=4 only'
        return out
    ref = json.load(open(f))
    err = _errors(_readouts(plain_chain, w.n), ref)
    d_ref = np.array(ref['discarded'])
    out['as_benchmarked'] = {
        'fixture': 'bench_n32_d20.json', 'max_err': err,
        'oracle_spread': {k: ref['conditioning'][k] for k in keys},
        'within_2x_spread': all(err[k] <= max(1e-5, 2 * ref['conditioning'][k]) for k in keys),
        'discarded_weight': {'per_bond_max_ref': float(d_ref.max()),
                             'max_err': float(np.abs(np.array(plain_disc) - d_ref).max())},
        'note': 'chi cap keeps rounding-level singular values and sqrt(S) splits lift them to sqrt(eps): '
                'complex128 oracle runs that differ only in rounding spread by the oracle_spread figures'}
    f2 = os.path.join(GOLDEN, 'bench_n32_d20_err1e-6.json')
    if os.path.exists(f2):
        ref2 = json.load(open(f2))
        disc = []
        ch = run_chain(ops, w, args.dtype, eng, max_err=1e-6, discarded=disc)
        err2 = _errors(_readouts(ch, w.n), ref2)
        floor = ref2.get('fp32_storage', {})
        out['well_conditioned'] = {
            'fixture': 'bench_n32_d20_err1e-6.json (max_truncation_err=1e-6)', 'max_err': err2,
            'oracle_spread': {k: ref2['conditioning'][k] for k in keys},
            'fp32_storage_floor': {k: floor.get(k) for k in keys},
            'dims_equal': [list(map(int, d)) for d in ch.dims()] == ref2['dims'],
            'discarded_weight_max_err': float(np.abs(np.array(disc) - np.array(ref2['discarded'])).max())}
        out['max_err'] = max(err2.values())
    return out


def grad_line(args, local):
    """grad-evals/s of the adjoint (mpdo_program_grad) on the hardware-efficient
    ansatz: n=24, 12 layers, chi=32, kappa=4, complex64; angles U[0, 2pi) from
    seed 0, depolarising p = 1e-3 per gate type; loss sum Z_i Z_{i+1} + 0.5
    sum X_i.  Each gradient is the forward pass with checkpoints, the readout
    adjoint and the reverse sweep (one recompute per truncate segment)."""
    import math
    import torch
    from mpdo_gb300 import Engine, adjoint as AD
    n, layers, chi, kappa = 24, 12, 32, 4
    g = torch.Generator().manual_seed(0)
    ang = (2 * math.pi * torch.rand(layers, 2, n, dtype=torch.float64, generator=g)).requires_grad_(True)
    p = {k: torch.tensor(1e-3, dtype=torch.float64, requires_grad=True) for k in ('ry', 'rz', 'cz')}
    eng = Engine.get(local)
    terms = AD.ising_terms(n)
    times, phases = [], []
    for k in range(args.grad_warmup + args.grad_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ang.grad = None
        for v in p.values():
            v.grad = None
        tm = {}
        loss = AD.program_loss(AD.hea_ops(ang, p), n, terms, chi, kappa, dtype='complex64', engine=eng, timing=tm)
        loss.backward()
        torch.cuda.synchronize()
        if k >= args.grad_warmup:
            times.append(time.perf_counter() - t0)
            phases.append(tm)
    ms = 1e3 * statistics.mean(times)
    ph = {k: statistics.mean(t[k] for t in phases) for k in phases[0]} if phases else {}
    return {'value': 1e3 / ms, 'unit': 'grad-evals/s', 'ms_per_grad': ms, 'steps': args.grad_steps,
            'warmup': args.grad_warmup, 'loss': float(loss), 'grad_norm_angles': float(ang.grad.norm()),
            'dloss_dp': {k: float(v.grad) for k, v in p.items()},
            'forward_ms': ph.get('forward_ms'), 'readout_ms': ph.get('readout_ms'),
            'reverse_ms': ph.get('reverse_ms'),
            'adjoint_over_forward': (ph['forward_ms'] + ph['readout_ms'] + ph['reverse_ms']) / ph['forward_ms']
            if ph else None,
            'config': {'workload': 'hardware-efficient ansatz: per layer RY and RZ on every qubit and a CZ ladder, '
                                   'each sublayer followed by truncate(); depolarising after every gate',
                       'n': n, 'layers': layers, 'angles': layers * 2 * n, 'noise_parameters': 3, 'chi': chi,
                       'kappa': kappa, 'dtype': 'c64',
                       'timing': 'wall clock around torch autograd (forward + backward) of the drop-in loss; '
                                 'phases by CUDA events inside the adjoint'}}


def gpu_arm(args):
    import numpy as np
    import torch
    rank, ws, local = dist_init(args)
    torch.cuda.set_device(local)
    import mpdo_gb300
    mpdo_gb300.build()
    from mpdo_gb300 import Batch, Engine
    import MPDOSimulator as S
    from mpdo_gb300.workloads import build_circuit
    peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))) if os.path.exists(
        os.path.join(ROOT, 'MEASURED_PEAKS.json')) else {}
    cdt = torch.complex64 if args.dtype == 'complex64' else torch.complex128
    B = max(1, args.batch)
    seeds = replica_seeds(rank, B)
    works = [workload(args, seed=s) for s in seeds]
    w = works[0]
    gates_per_circuit = w.gates
    device = f'cuda:{local}'
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device='cuda')   # 256 MB > L2
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    # ---- engine options: built-in defaults, or the autotuner's for this class
    tuning = {'source': 'defaults'}
    if args.autotune:
        from mpdo_gb300 import autotune
        opts = autotune.options_for(w.chi, w.kappa, args.dtype, local)
        tuning = {'source': 'cache', 'options': opts}
        if not opts:
            ent = autotune.tune(w.chi, w.kappa, args.dtype, local)
            opts = ent['options']
            tuning = {'source': 'tuned before the run', 'options': opts, 'seconds': ent['seconds'],
                      'default_seconds': ent['default_seconds']}
        autotune.apply(Engine.get(local), opts)
        autotune.apply(Batch.get(local, args.workers), opts)

    # ---- plain path: one circuit through one engine (device-resident inputs)
    eng = Engine.get(local)
    eng.set_stream(stream.cuda_stream)
    circuit, ops = host_ops(w, args.dtype, device)
    for _ in range(args.plain_warmup):
        run_chain(ops, w, args.dtype, eng)
    torch.cuda.synchronize()
    plain_ms = []
    for _ in range(args.plain_steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run_chain(ops, w, args.dtype, eng)
        b.record(stream)
        b.synchronize()
        plain_ms.append(a.elapsed_time(b))
    eng.sync()
    eng.profile(True)
    plain_disc = []
    plain_chain = run_chain(ops, w, args.dtype, eng, discarded=plain_disc)
    plain_prof = eng.profile_read()
    eng.profile(False)
    plain_wide = plain_prof.pop('wide_bonds')
    plain_phases = plain_prof.pop('phases')
    t0 = time.perf_counter()
    circuit.evolve(S.Tools.create_ket0Series(w.n, dtype=cdt, connected=True))
    marg = circuit.probabilities([0])
    torch.cuda.synchronize()
    plain_e2e_ms = 1e3 * (time.perf_counter() - t0)
    dw = [np.asarray(d, dtype=np.float64).ravel() for d in plain_disc if d is not None]
    plain = {'value': gates_per_circuit / (statistics.mean(plain_ms) / 1e3), 'unit': 'gates/s',
             'ms_per_circuit': statistics.mean(plain_ms), 'steps': args.plain_steps, 'warmup': args.plain_warmup,
             'e2e_value': gates_per_circuit / (plain_e2e_ms / 1e3), 'e2e_ms': plain_e2e_ms,
             'roofline': _roofline(plain_prof, peaks),
             'kernel_breakdown_ms': {k: {'launches': v['launches'], 'ms': round(v['ms'], 3)}
                                     for k, v in plain_prof.items() if v['launches']},
             'wide_bond_svd': plain_wide,
             'phases_ms': {k: round(v['ms'], 1) for k, v in plain_phases.items()},
             'discarded_weight': {'per_bond_max': max((float(d.max()) for d in dw if d.size), default=None),
                                  'last_truncation_sum': float(dw[-1].sum()) if dw else None,
                                  'truncations': len(dw)},
             'marginal_q0': [float(x) for x in marg.tolist()]}
    par = None
    if rank == 0 and not args.no_parity:
        par = parity(args, w, ops, eng, plain_chain, plain_disc)
    del plain_chain
    eng.set_stream(None)

    # ---- batched: B independent circuits (seeds) on W worker engines
    batch = Batch.get(local, args.workers)
    progs = [program(wk, host_ops(wk, args.dtype, device)[1], args.dtype) for wk in works]
    for _ in range(args.warmup):
        batch.run(progs)
    torch.cuda.synchronize()
    barrier(ws)
    launches0 = eng.launch_count()
    hist0 = eng.launch_histogram()
    step_ms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            stream.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            res = batch.run(progs)          # returns once every worker engine has synchronised
            b.record(stream)
            b.synchronize()
            step_ms.append(a.elapsed_time(b))
    barrier(ws)
    launches = eng.launch_count() - launches0
    hist1 = eng.launch_histogram()
    by_launcher = {k: (v - hist0.get(k, 0)) // args.steps for k, v in hist1.items() if v - hist0.get(k, 0)}
    clocks = clk.summary()
    total_ms = allreduce_max(sum(step_ms), ws)
    value = ws * B * gates_per_circuit * args.steps / (total_ms / 1e3)
    for e in batch.engines:
        e.profile(True)
    batch.run(progs)
    bprofs = [e.profile_read() for e in batch.engines]
    for e in batch.engines:
        e.profile(False)
    bprof = _sum_profiles(bprofs)
    wide = {'range_finder': sum(p['wide_bonds']['range_finder'] for p in bprofs),
            'exact': sum(p['wide_bonds']['exact'] for p in bprofs)}

    # ---- batched e2e: the public API with host inputs and host results
    e2e_ms = []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cs = [build_circuit(wk, dtype=cdt, device=device) for wk in works]
        out = S.evolve_batch(cs, [S.Tools.create_ket0Series(wk.n, dtype=cdt, connected=True) for wk in works],
                             workers=args.workers)
        zs = [np.asarray(r['z']) for r in out]
        torch.cuda.synchronize()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_total = allreduce_max(sum(e2e_ms), ws)
    e2e_value = ws * B * gates_per_circuit * len(e2e_ms) / (e2e_total / 1e3)
    h2d = sum(sum(op[2].size * 16 for op in p['ops'] if len(op) > 2) + w.n * 32 for p in progs)
    d2h = B * 8 * (w.n + (w.n - 1) + (w.n - 1) * w.gate_layers)

    # ---- the adjoint: grad-evals/s
    grad = grad_line(args, local) if args.grad_steps > 0 and rank == 0 else None
    if rank != 0:
        return
    # seed 0's batch readouts against the oracle (the batched path gives <Z>, <ZZ>)
    if par is not None and 'as_benchmarked' in par:
        ref = json.load(open(os.path.join(GOLDEN, 'bench_n32_d20.json')))
        par['as_benchmarked']['batched_seed0_max_err'] = {
            'z': float(np.abs(np.asarray(res[0]['z']) - ref['z']).max()),
            'zz': float(np.abs(np.asarray(res[0]['zz']) - ref['zz']).max())}
    ref_flops, _ = reference_trace_flops(w)
    step_s = total_ms / args.steps / 1e3
    ref_rate = B * ref_flops / step_s / 1e12
    bf16 = peaks.get('bf16_tflops')
    z0 = [float(x) for x in zs[0][:4]]
    out = {'metric': METRIC, 'value': value, 'unit': 'gates/s', 'n_gpus': ws, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': total_ms / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'c64' if args.dtype == 'complex64' else 'c128', 'data': 'synthetic',
           'config': {'workload': f'{B} independent circuits of {w.name}, seeds {seeds[0]}..{seeds[-1]}',
                      'n': w.n, 'depth': w.depth, 'chi': w.chi, 'kappa': w.kappa, 'circuits_per_step': B,
                      'workers': batch.workers, 'gates_per_circuit': gates_per_circuit,
                      'gate_layers_per_circuit': w.gate_layers, 'parallelism': f'replicas{ws}',
                      'l2': 'flushed between steps (256 MB write); the per-circuit state is ~8 MB',
                      'engine_options': tuning,
                      'timing': 'CUDA events on an idle stream around the synchronous batch call'},
           'e2e': {'value': e2e_value, 'unit': 'gates/s', 'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': d2h,
                   'ms_per_step': e2e_total / len(e2e_ms),
                   'path': 'MPDOSimulator.evolve_batch on TensorCircuit objects built per step'},
           'gpu_launches': int(launches),
           'gpu_launches_per_step_by_launcher': dict(sorted(by_launcher.items(), key=lambda kv: -kv[1])),
           'clocks': clocks, 'roofline': _roofline(bprof, peaks),
           'roofline_reference_trace': {
               'achieved': ref_rate, 'unit': 'TFLOP/s', 'peak_fp32_simt_nominal': FP32_SIMT_NOMINAL_TFLOPS,
               'frac_of_fp32_simt_nominal': ref_rate / FP32_SIMT_NOMINAL_TFLOPS,
               'peak_bf16_tensor_measured': bf16, 'frac_of_measured_bf16_tensor': ref_rate / bf16 if bf16 else None,
               'flops_per_circuit': ref_flops,
               'how': "the reference algorithm's flops on this circuit from its shape trace (SVDs of the contracted "
                      'pairs, QRs, kappa SVDs, contractions; 8d formulas) per step over the step time; the engine '
                      'does less work than that (its isometry shortcut decomposes one site per bond)'},
           'kernel_breakdown_ms': {k: {'launches': v['launches'], 'ms': round(v['ms'], 3)}
                                   for k, v in bprof.items() if v['launches']},
           'wide_bond_svd': wide, 'z_first_circuit': z0,
           'parity': par, 'grad': grad,
           'plain': plain, 'batched_over_plain': value / plain['value']}
    print('gpu part: ' + json.dumps(out), file=sys.stderr, flush=True)
    if ws == 1 and not args.no_cpu_baseline:
        cpu = CpuLayer(w, threads=os.cpu_count())
        v, secs = cpu.sample()
        out['cpu_baseline'] = {'value': v, 'unit': 'gates/s', 'cores': cpu.threads, 'kind': 'port',
                               'sample': cpu.describe() + f'; {secs:.1f} s for the layer'}
    print(json.dumps(out), flush=True)


def uneven_circuits(rank, ws, count):
    """This rank's circuits of the uneven batch (seeds 0..count-1): the
    longest-processing-time split of their reference-trace flops over ws
    ranks.  Returns (seeds, per-rank estimated flops, imbalance)."""
    from mpdo_gb300.schedule import imbalance, partition, reference_flops
    from mpdo_gb300.workloads import uneven_batch_circuit
    costs = [reference_flops(uneven_batch_circuit(s))[0] for s in range(count)]
    parts = partition(costs, ws)
    return parts[rank], [sum(costs[i] for i in p) for p in parts], imbalance(parts, costs)


def uneven_arm(args):
    """The uneven batch: circuits with n ~ U{12..40}, depth ~ U{10..30},
    chi from {16, 32, 64, 128}, kappa from {2, 4} (workloads.uneven_batch_circuit),
    complex64.  One step evolves this rank's share of them through the batch
    runner; value = gate layers of all ranks' circuits per second (max time
    over ranks).  --sequential also runs this rank's circuits one at a time
    through one engine (the plain path), timed in full, for the ratio."""
    import torch
    rank, ws, local = dist_init(args)
    torch.cuda.set_device(local)
    import mpdo_gb300
    mpdo_gb300.build()
    from mpdo_gb300 import Batch, Engine
    from mpdo_gb300.workloads import uneven_batch_circuit
    seeds, rank_flops, imb = uneven_circuits(rank, ws, args.circuits)
    works = [uneven_batch_circuit(s) for s in seeds]
    device = f'cuda:{local}'
    progs = [program(w, host_ops(w, args.dtype, device)[1], args.dtype) for w in works]
    layers = sum(w.gate_layers for w in works)
    gates = sum(w.gates for w in works)
    batch = Batch.get(local, args.workers)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device='cuda')
    # warm-up: --warmup whole batches, or with --warmup 0 the 16 costliest
    # circuits once (each step is minutes of work)
    for _ in range(args.warmup):
        batch.run(progs)
    if args.warmup == 0:
        batch.run(progs[:16])
    torch.cuda.synchronize()
    barrier(ws)
    step_ms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            batch.run(progs)
            b.record()
            b.synchronize()
            step_ms.append(a.elapsed_time(b))
    barrier(ws)
    clocks = clk.summary()
    total_ms = allreduce_max(sum(step_ms), ws)
    all_layers = allreduce_sum(layers, ws)
    all_gates = allreduce_sum(gates, ws)
    value = all_layers * args.steps / (total_ms / 1e3)
    print(f'uneven batch: {total_ms / args.steps / 1e3:.1f} s per step, {value:.1f} gate-layers/s', file=sys.stderr,
          flush=True)
    seq = None
    if args.sequential:
        eng = Engine.get(local)
        t_seq = []
        for w, p in zip(works, progs):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ch = run_chain(p['ops'], w, args.dtype, eng)
            eng.sync()
            t_seq.append(time.perf_counter() - t0)
            del ch
            print(f'sequential: {w.name}: {t_seq[-1]:.2f} s ({len(t_seq)}/{len(works)}, {sum(t_seq):.1f} s so far)',
                  file=sys.stderr, flush=True)
        seq_s = allreduce_max(sum(t_seq), ws)
        seq = {'value': all_layers / seq_s, 'unit': 'gate-layers/s', 'seconds': seq_s,
               'path': 'the same circuits one at a time through one engine (Chain ops), wall clock',
               'slowest_circuit_s': max(t_seq)}
    if rank != 0:
        return
    chis = {}
    for w in works:
        chis[w.chi] = chis.get(w.chi, 0) + 1
    out = {'metric': 'gate-layers/s, uneven batch (256 circuits)', 'value': value, 'unit': 'gate-layers/s',
           'n_gpus': ws, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': total_ms / args.steps,
           'higher_is_better': True, 'scaling': 'strong', 'vs_baseline': None, 'dtype': 'c64',
           'data': 'synthetic',
           'config': {'workload': f'uneven batch, seeds 0..{args.circuits - 1}: n ~ U{{12..40}}, depth ~ '
                                  'U{10..30}, chi in {16, 32, 64, 128}, kappa in {2, 4}, U3 + CZ/CNOT brickwork '
                                  'with the n=32 workload noise',
                      'circuits': args.circuits, 'circuits_this_rank': len(works), 'chi_histogram': chis,
                      'gate_layers': all_layers, 'gates': all_gates, 'workers': batch.workers,
                      'l2': 'flushed before each step; each step is ~minutes of work',
                      'partition': {'rule': 'longest processing time first on the reference-trace flops',
                                    'rank_flops': rank_flops, 'imbalance': imb,
                                    'measured_on_hardware': ws > 1}},
           'gates_per_s': all_gates * args.steps / (total_ms / 1e3), 'clocks': clocks,
           'warmup_rule': 'whole batches' if args.warmup else 'the 16 costliest circuits once',
           'sequential_plain': seq, 'batched_over_sequential': value / seq['value'] if seq else None}
    print(json.dumps(out), flush=True)


def allreduce_sum(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device='cuda' if dist.get_backend() == 'nccl' else 'cpu')
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def main():
    args = parse()
    if args.impl == 'reference':
        reference_arm(args)
    elif args.workload == 'uneven':
        uneven_arm(args)
    else:
        gpu_arm(args)


if __name__ == '__main__':
    main()
