#!/usr/bin/env python
"""Benchmark of the MPDO noisy-circuit hot path (gates/s).

Workload (default): n=32 qubits, depth 20 (U3 on every qubit, then CZ/CNOT
brickwork, seed 0), 1q depolarising 1e-3 + amplitude damping 1e-3 after every
1q gate, 2q depolarising 1e-2 after every 2q gate, a truncate() after every
sublayer, chi=64, kappa=4, complex64.  One step = one full evolution of that
circuit (960 gates, 40 truncate layers).

value: gates/s with the circuit's Kraus tensors prepared on the host and the
       state created on the device, CUDA events on the engine's stream around
       the K timed steps (L2 flushed between steps).
e2e:   the same through the drop-in API (TensorCircuit.evolve from a host
       product state, then a device->host read of a single-qubit marginal).
roofline: per-kernel-class CUDA-event timing of one extra step; the dominant
       class's algorithmic flops (or bytes) / its time against the measured peak.
cpu_baseline / --impl reference: the CPU oracle (restatement of the reference
       path, torch CPU, exact SVD) on a steady-state layer of the same circuit.

Multi-GPU (torchrun, N > 1): independent replicas of the circuit, one per GPU
(the path does not shard within a circuit); value = total gates / max time.
"""
import argparse
import json
import os
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

METRIC = json.load(open(os.path.join(ROOT, 'BASELINE.json')))['metric']
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
def workload(args):
    from mpdo_gb300.workloads import config1
    return config1(n=args.n, depth=args.depth, chi=args.chi, kappa=args.kappa)


def host_ops(w, dtype):
    """Kraus tensors of every gate, built by the drop-in API's own builders."""
    import numpy as np
    import torch
    from mpdo_gb300.workloads import build_circuit
    c = build_circuit(w, dtype=torch.complex64 if dtype == 'complex64' else torch.complex128, device='cuda:0')
    ops = []
    for i, layer in enumerate(c.layers):
        name = layer.name.lower()
        if 'truncate' in name:
            ops.append(('t',))
            continue
        oqs = c._oqs_list[i]
        if layer.single:
            ops.append(('1', oqs[0], np.ascontiguousarray(c._noisy_1q(layer))))
        else:
            t = c._noisy_2q(layer)
            if t.ndim == 4:
                t = t[..., None]
            a, b = oqs
            if a > b:
                t = np.transpose(t, (1, 0, 3, 2, 4))
            ops.append(('2', min(a, b), np.ascontiguousarray(t)))
    return c, ops


def run_chain(ops, w, dtype, eng):
    from mpdo_gb300 import Chain
    ch = Chain([[1, 0]] * w.n, dtype=dtype, connected=True, engine=eng)
    for op in ops:
        if op[0] == '1':
            ch.apply_1q(op[1], op[2])
        elif op[0] == '2':
            ch.apply_2q(op[1], op[2], 2.718281828459045e-8)
        else:
            ch.truncate(w.chi, w.kappa, None, True)
    return ch


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
def cpu_layer(w, budget_s, threads=None):
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
    O.evolve(st, layers[0], chi=w.chi, kappa=w.kappa, noisy=True)
    secs, info = O.time_layer(st, layers[1], w.chi, w.kappa, budget_s=budget_s)
    gates = sum(1 for op in layers[1] if op[0] != 'truncate')
    return gates / secs, gates, secs, info, torch.get_num_threads()


def reference_arm(args):
    rank, ws, _ = dist_init(args)
    if rank != 0:
        return
    import torch
    w = workload(args)
    cores = os.cpu_count() or 1
    vals = []
    for k in range(args.warmup + args.steps):
        v, gates, secs, info, th = cpu_layer(w, args.cpu_budget / max(1, args.steps), threads=cores)
        if k >= args.warmup:
            vals.append(v)
        if k + 1 >= args.warmup and args.warmup > 1:
            pass
    # warm-up steps are cheap repeats of the same sample; the timed value is the mean
    val = sum(vals) / len(vals)
    sample = (f'steady-state layer 1 of the workload ({gates} gates) on the CPU oracle, torch {torch.__version__}, '
              f'{th} threads, exact SVD; {info["extrapolated_svd_steps"]} of '
              f'{info["extrapolated_svd_steps"] + info["measured_svd_steps"]} SVD-sweep steps extrapolated')
    out = {'metric': METRIC, 'value': val, 'unit': 'gates/s', 'n_gpus': args.gpus, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': 1e3 * gates / val, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic', 'impl': 'reference',
           'config': {'workload': w.name, 'n': w.n, 'depth': w.depth, 'chi': w.chi, 'kappa': w.kappa,
                      'step': 'one steady-state layer (sample)'},
           'cpu_baseline': {'value': val, 'unit': 'gates/s', 'cores': th, 'kind': 'port', 'sample': sample},
           'e2e': {'value': val, 'unit': 'gates/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------- GPU arm --
def gpu_arm(args):
    import numpy as np
    import torch
    rank, ws, local = dist_init(args)
    torch.cuda.set_device(local)
    import mpdo_gb300
    mpdo_gb300.build()
    from mpdo_gb300 import Engine
    import MPDOSimulator as S
    eng = Engine.get(local)
    # one explicit stream shared by torch (events, L2 flush) and the engine
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)
    w = workload(args)
    circuit, ops = host_ops(w, args.dtype)
    gates_per_step = w.gates

    # warm-up
    for _ in range(args.warmup):
        run_chain(ops, w, args.dtype, eng)
    torch.cuda.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device='cuda')   # 256 MB > L2

    # ---- value: device-resident inputs, CUDA events on the engine stream
    barrier(ws)
    torch.cuda.synchronize()
    launches0 = eng.launch_count()
    evs = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ch = run_chain(ops, w, args.dtype, eng)
            b.record(stream)
            evs.append((a, b, ch))
        torch.cuda.synchronize()
    barrier(ws)
    launches = eng.launch_count() - launches0
    eng.sync()
    step_ms = [a.elapsed_time(b) for a, b, _ in evs]
    total_ms = allreduce_max(sum(step_ms), ws)
    value = ws * gates_per_step * args.steps / (total_ms / 1e3)
    clocks = clk.summary()

    # ---- e2e: public API with host buffers
    dtype = torch.complex64 if args.dtype == 'complex64' else torch.complex128
    e2e_ms = []
    for k in range(args.steps + 1):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        state = S.Tools.create_ket0Series(w.n, dtype=dtype, connected=True)
        circuit.evolve(state)
        marg = circuit.probabilities([0])
        torch.cuda.synchronize()
        if k > 0:
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_total = allreduce_max(sum(e2e_ms), ws)
    dw = [np.asarray(d, dtype=np.float64).ravel() for d in circuit.discarded_weights if d is not None]
    e2e_value = ws * gates_per_step * len(e2e_ms) / (e2e_total / 1e3)
    esz = 8 if args.dtype == 'complex64' else 16
    h2d = w.n * 2 * esz + sum(op[2].size * 16 for op in ops if op[0] != 't')      # vectors + Kraus parameters
    d2h = 8 * 2 + 8 * (w.n - 1) * w.gate_layers                                   # marginal + discarded weights

    # ---- roofline: one profiled step
    eng.profile(True)
    run_chain(ops, w, args.dtype, eng)
    prof = eng.profile_read()
    eng.profile(False)
    wide = prof.pop('wide_bonds')
    dom = max(prof, key=lambda k: prof[k]['ms'])
    d = prof[dom]
    peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))) if os.path.exists(
        os.path.join(ROOT, 'MEASURED_PEAKS.json')) else {}
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
                 'launches_per_step': d['launches'], 'ms_per_step': d['ms'], 'share_of_step': d['ms'] / (sum(
                     v['ms'] for v in prof.values()) or 1), 'algorithmic_per_launch': per_launch_alg,
                 'traffic': None})
    tfile = os.path.join(ROOT, 'profiles', 'traffic.json')
    if os.path.exists(tfile):
        tr = json.load(open(tfile)).get(dom)
        if tr:
            roof['traffic'] = tr.get('bytes_per_launch')
    breakdown = {k: {'launches': v['launches'], 'ms': round(v['ms'], 3)} for k, v in prof.items() if v['launches']}

    if rank != 0:
        return
    out = {'metric': METRIC, 'value': value, 'unit': 'gates/s', 'n_gpus': ws, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': total_ms / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'c64' if args.dtype == 'complex64' else 'c128', 'data': 'synthetic',
           'config': {'workload': w.name, 'n': w.n, 'depth': w.depth, 'chi': w.chi, 'kappa': w.kappa,
                      'gates_per_step': gates_per_step, 'gate_layers_per_step': w.gate_layers,
                      'parallelism': f'replicas{ws}', 'l2': 'flushed between steps (256 MB write)'},
           'e2e': {'value': e2e_value, 'unit': 'gates/s', 'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': d2h,
                   'ms_per_step': e2e_total / len(e2e_ms)},
           'gpu_launches': int(launches), 'clocks': clocks, 'roofline': roof, 'kernel_breakdown_ms': breakdown,
           'wide_bond_svd': wide,
           'discarded_weight': {'per_bond_max': max((float(d.max()) for d in dw if d.size), default=None),
                                'last_truncation_sum': float(dw[-1].sum()) if dw else None,
                                'truncations': len(dw)},
           'marginal_q0': [float(x) for x in marg.tolist()]}
    print('gpu part: ' + json.dumps(out), file=sys.stderr, flush=True)
    if ws == 1 and not args.no_cpu_baseline:
        v, gates, secs, info, th = cpu_layer(w, args.cpu_budget, threads=os.cpu_count())
        out['cpu_baseline'] = {'value': v, 'unit': 'gates/s', 'cores': th, 'kind': 'port',
                               'sample': f'steady-state layer 1 ({gates} gates) of the same circuit on the CPU oracle '
                                         f'(torch CPU, exact SVD), {info["extrapolated_svd_steps"]} of '
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
