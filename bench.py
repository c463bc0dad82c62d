#!/usr/bin/env python
"""Benchmark of the MPDO noisy-circuit hot path (gates/s).

Circuit (the n=32, chi=64, kappa=4 workload): 32 qubits, depth 20 (U3 on every
qubit, then CZ/CNOT brickwork), 1q depolarising 1e-3 + amplitude damping 1e-3
after every 1q gate, 2q depolarising 1e-2 after every 2q gate, a truncate()
after every sublayer, complex64; 950 gates and 40 truncate layers.

One step = one batch of --batch independent circuits of that shape (seeds
0..B-1) through the batched engine (--workers worker engines, each with its
own stream and memory pool).
value: gates/s over the K timed steps, CUDA events on an idle stream around
       the synchronous batch call (Kraus tensors are host data by design: they
       travel as kernel parameters), L2 flushed between steps.
e2e:   the same circuits through the public API (MPDOSimulator.evolve_batch on
       TensorCircuit objects built per step, host product states in, <Z_i>,
       <Z_i Z_i+1> and per-bond discarded weights out).
plain: one circuit through one engine (CUDA events on its stream) and through
       TensorCircuit.evolve, with its own roofline and kernel breakdown.
roofline: per-kernel-class CUDA-event timing of one extra batch; the dominant
       class's algorithmic flops (or bytes) / its summed launch time against
       the measured peak.
cpu_baseline / --impl reference: the CPU oracle (restatement of the reference
       path, torch CPU, with the reference's randomized SVD for capped SVDs
       of >= 1e4 elements) on a steady-state layer of the seed-0
       circuit (the reference evolves circuits one after another).

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
    ap.add_argument('--cpu-budget', type=float, default=20.0, help='seconds of CPU work for the baseline sample')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--batch', type=int, default=24, help='independent circuits per step (seeds)')
    ap.add_argument('--workers', type=int, default=24, help='worker engines of the batch runner')
    ap.add_argument('--plain-steps', type=int, default=1, help='timed single-circuit runs (reported as plain)')
    ap.add_argument('--plain-warmup', type=int, default=1)
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


def host_ops(w, dtype):
    """The circuit as the drop-in API builds it and the engine operations its
    evolve() performs (Kraus tensors by the API's own builders)."""
    import torch
    from mpdo_gb300.workloads import build_circuit
    c = build_circuit(w, dtype=torch.complex64 if dtype == 'complex64' else torch.complex128, device='cuda:0')
    return c, c._engine_ops()


def run_chain(ops, w, dtype, eng):
    from mpdo_gb300 import Chain
    ch = Chain([[1, 0]] * w.n, dtype=dtype, connected=True, engine=eng)
    for op in ops:
        if op[0] == '1q':
            ch.apply_1q(op[1], op[2])
        elif op[0] == '2q':
            ch.apply_2q(op[1], op[2], 2.718281828459045e-8)
        elif op[0] == 'truncate':
            ch.truncate(w.chi, w.kappa, None, True)
        else:
            ch.kappa_truncate(w.kappa, None)
    return ch


def program(w, ops, dtype):
    return dict(n=w.n, dtype=dtype, vectors=[[1, 0]] * w.n, connected=True, chi=w.chi, kappa=w.kappa,
                max_err=None, noisy=True, ops=ops, z=True, zz=True, discarded=True)


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
def cpu_layer(w, budget_s, threads=None, randomized=True):
    """Gates/s of the CPU oracle on a steady-state layer of the workload:
    layer 0 runs in full (bonds reach chi), layer 1 is timed with the SVD
    sweep extrapolated past the budget.  Factorisations in complex128 with the
    state stored in complex64 (the Arm hosts' LAPACK aborts on some complex64
    SVDs)."""
    import torch
    from oracle import mpdo_oracle as O
    if threads:
        torch.set_num_threads(threads)
    dt = torch.complex64
    dec = O.amplitude_damping(w.noise['gamma'], dt)
    dep = O.depolarization(w.noise['p1'], 1, dt)
    dp2 = O.depolarization(w.noise['p2'], 2, dt)
    layers, cur = [], []
    subs = 0
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
    st = O.product_state([[1, 0]] * w.n, connected=True, dtype=dt)
    # the reference's stock SVD: its vendored backend switches capped SVDs of
    # >= 1e4 elements to a randomized SVD (decompositions.py:112-115)
    O.evolve(st, layers[0], chi=w.chi, kappa=w.kappa, noisy=True, randomized=randomized)
    secs, info = O.time_layer(st, layers[1], w.chi, w.kappa, budget_s=budget_s, randomized=randomized)
    info['svd'] = ('SVDs as the reference takes them (randomized for capped matrices of >= 1e4 elements, exact '
                   'otherwise)' if randomized else 'every SVD exact')
    gates = sum(1 for op in layers[1] if op[0] != 'truncate')
    return gates / secs, gates, secs, info, torch.get_num_threads()


def cpu_layer_any(w, budget_s, threads=None):
    """``cpu_layer`` with the reference's randomized branch; should that
    branch fail on this host's LAPACK, the sample is retaken with exact SVDs
    and says so."""
    try:
        return cpu_layer(w, budget_s, threads, randomized=True)
    except Exception as e:  # noqa: BLE001 -- reported in the sample text
        out = cpu_layer(w, budget_s, threads, randomized=False)
        out[3]['svd'] += f' (the randomized branch failed here: {type(e).__name__}: {e})'
        return out


def reference_arm(args):
    rank, ws, _ = dist_init(args)
    if rank != 0:
        return
    import torch
    w = workload(args)
    cores = os.cpu_count() or 1
    vals = []
    for k in range(args.warmup + args.steps):
        v, gates, secs, info, th = cpu_layer_any(w, args.cpu_budget / max(1, args.steps), threads=cores)
        if k >= args.warmup:
            vals.append(v)
        if k + 1 >= args.warmup and args.warmup > 1:
            pass
    # warm-up steps are cheap repeats of the same sample; the timed value is the mean
    val = sum(vals) / len(vals)
    sample = (f'steady-state layer 1 of the workload ({gates} gates) on the CPU oracle, torch {torch.__version__}, '
              f'{th} threads, {info["svd"]}; {info["extrapolated_svd_steps"]} of '
              f'{info["extrapolated_svd_steps"] + info["measured_svd_steps"]} SVD-sweep steps extrapolated')
    out = {'metric': METRIC, 'value': val, 'unit': 'gates/s', 'n_gpus': args.gpus, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': 1e3 * gates / val, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic', 'impl': 'reference',
           'config': {'workload': f'{max(1, args.batch)} independent circuits of {w.name}, seeds 0..'
                                  f'{max(1, args.batch) - 1}', 'n': w.n, 'depth': w.depth, 'chi': w.chi,
                      'kappa': w.kappa, 'circuits_per_step': max(1, args.batch),
                      'step': 'circuits run one after another; each step times a sample: one steady-state '
                              'layer of the seed-0 circuit'},
           'cpu_baseline': {'value': val, 'unit': 'gates/s', 'cores': th, 'kind': 'port', 'sample': sample},
           'e2e': {'value': val, 'unit': 'gates/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------- GPU arm --
def _roofline(prof, peaks):
    dom = max(prof, key=lambda k: prof[k]['ms'])
    d = prof[dom]
    if dom in ('kraus1q', 'mix2q', 'other'):
        achieved = d['bytes'] / (d['ms'] / 1e3) / 1e9
        peak = peaks.get('hbm_gbs', 6800.0)
        roof = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak}
        per_launch_alg = d['bytes'] / max(1, d['launches'])
    else:
        achieved = d['flops'] / (d['ms'] / 1e3) / 1e12
        peak = peaks.get('bf16_tflops', 1900.0)
        roof = {'bound': 'tensor', 'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s', 'frac': achieved / peak,
                'frac_of_fp32_simt_nominal': achieved / FP32_SIMT_NOMINAL_TFLOPS}
        per_launch_alg = d['flops'] / max(1, d['launches'])
    roof.update({'kernel': dom, 'peak_source': 'measured (MEASURED_PEAKS.json)' if peaks else 'fallback',
                 'launches': d['launches'], 'kernel_ms': d['ms'],
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
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device='cuda')   # 256 MB > L2
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    # ---- plain path: one circuit through one engine (device-resident inputs)
    eng = Engine.get(local)
    eng.set_stream(stream.cuda_stream)
    circuit, ops = host_ops(w, args.dtype)
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
    run_chain(ops, w, args.dtype, eng)
    plain_prof = eng.profile_read()
    eng.profile(False)
    plain_wide = plain_prof.pop('wide_bonds')
    plain_phases = plain_prof.pop('phases')
    t0 = time.perf_counter()
    circuit.evolve(S.Tools.create_ket0Series(w.n, dtype=cdt, connected=True))
    marg = circuit.probabilities([0])
    torch.cuda.synchronize()
    plain_e2e_ms = 1e3 * (time.perf_counter() - t0)
    dw = [np.asarray(d, dtype=np.float64).ravel() for d in circuit.discarded_weights if d is not None]
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
    eng.set_stream(None)

    # ---- batched: B independent circuits (seeds) on W worker engines
    batch = Batch.get(local, args.workers)
    progs = [program(wk, host_ops(wk, args.dtype)[1], args.dtype) for wk in works]
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
        cs = [build_circuit(wk, dtype=cdt, device=f'cuda:{local}') for wk in works]
        out = S.evolve_batch(cs, [S.Tools.create_ket0Series(wk.n, dtype=cdt, connected=True) for wk in works],
                             workers=args.workers)
        zs = [np.asarray(r['z']) for r in out]
        torch.cuda.synchronize()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_total = allreduce_max(sum(e2e_ms), ws)
    e2e_value = ws * B * gates_per_circuit * len(e2e_ms) / (e2e_total / 1e3)
    h2d = sum(sum(op[2].size * 16 for op in p['ops'] if len(op) > 2) + w.n * 32 for p in progs)
    d2h = B * 8 * (w.n + (w.n - 1) + (w.n - 1) * w.gate_layers)
    if rank != 0:
        return
    z0 = [float(x) for x in zs[0][:4]]
    out = {'metric': METRIC, 'value': value, 'unit': 'gates/s', 'n_gpus': ws, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': total_ms / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'c64' if args.dtype == 'complex64' else 'c128', 'data': 'synthetic',
           'config': {'workload': f'{B} independent circuits of {w.name}, seeds {seeds[0]}..{seeds[-1]}',
                      'n': w.n, 'depth': w.depth, 'chi': w.chi, 'kappa': w.kappa, 'circuits_per_step': B,
                      'workers': batch.workers, 'gates_per_circuit': gates_per_circuit,
                      'gate_layers_per_circuit': w.gate_layers, 'parallelism': f'replicas{ws}',
                      'l2': 'flushed between steps (256 MB write); the per-circuit state is ~8 MB',
                      'timing': 'CUDA events on an idle stream around the synchronous batch call'},
           'e2e': {'value': e2e_value, 'unit': 'gates/s', 'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': d2h,
                   'ms_per_step': e2e_total / len(e2e_ms),
                   'path': 'MPDOSimulator.evolve_batch on TensorCircuit objects built per step'},
           'gpu_launches': int(launches),
           'gpu_launches_per_step_by_launcher': dict(sorted(by_launcher.items(), key=lambda kv: -kv[1])),
           'clocks': clocks, 'roofline': _roofline(bprof, peaks),
           'kernel_breakdown_ms': {k: {'launches': v['launches'], 'ms': round(v['ms'], 3)}
                                   for k, v in bprof.items() if v['launches']},
           'wide_bond_svd': wide, 'z_first_circuit': z0,
           'plain': plain, 'batched_over_plain': value / plain['value']}
    print('gpu part: ' + json.dumps(out), file=sys.stderr, flush=True)
    if ws == 1 and not args.no_cpu_baseline:
        v, gates, secs, info, th = cpu_layer_any(w, args.cpu_budget, threads=os.cpu_count())
        out['cpu_baseline'] = {'value': v, 'unit': 'gates/s', 'cores': th, 'kind': 'port',
                               'sample': f'steady-state layer 1 ({gates} gates) of the seed-0 circuit on the CPU '
                                         f'oracle (torch CPU, {info["svd"]}), {info["extrapolated_svd_steps"]} of '
                                         f'{info["extrapolated_svd_steps"] + info["measured_svd_steps"]} SVD-sweep '
                                         f'steps extrapolated from measured ones; est. {secs:.1f} s per layer'}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == 'reference':
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == '__main__':
    main()
