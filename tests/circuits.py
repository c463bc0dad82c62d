"""Seeded test circuits as oracle op lists (Kraus tensors from the oracle's
own restatement of the reference's gate and noise builders)."""
import math
import random


from oracle import mpdo_oracle as O


def noise_cfg(p1=1e-3, gamma=1e-3, p2=1e-2):
    return dict(decay=O.amplitude_damping(gamma), dephasing=O.depolarization(p1),
                dpc2=O.depolarization(p2, 2))


def brickwork(n, layers, seed=0, noisy=True, gates2=('CNOT', 'CZ'), one_q=('RY', 'RZ'), nz=None):
    """1q sublayers (each followed by truncate) then a 2q brickwork sublayer."""
    nz = nz or noise_cfg()
    rng = random.Random(seed)
    ops = []
    for L in range(layers):
        for name in one_q:
            for q in range(n):
                if name == 'U3':
                    g = O.gate_1q('U3', *(rng.random() * 2 * math.pi for _ in range(3)))
                else:
                    g = O.gate_1q(name, rng.random() * 2 * math.pi)
                ops.append(('1q', q, O.noisy_1q(nz['decay'], nz['dephasing'], g) if noisy else g))
            ops.append(('truncate',))
        for q in range(L % 2, n - 1, 2):
            g = O.gate_2q(rng.choice(gates2))
            if rng.random() < 0.3:
                ops.append(('2q', q + 1, q, O.noisy_2q(nz['dpc2'], g) if noisy else g))
            else:
                ops.append(('2q', q, q + 1, O.noisy_2q(nz['dpc2'], g) if noisy else g))
        ops.append(('truncate',))
    return ops


def run_engine(chain, ops, chi, kappa, max_err=None, noisy=True, cutoff=O.GLOBAL_MINIMUM):
    last = None
    for op in ops:
        if op[0] == '1q':
            chain.apply_1q(op[1], op[2].numpy())
        elif op[0] == '2q':
            i, t = O.orient_2q(op[1], op[2], op[3])
            chain.apply_2q(i, t.numpy(), cutoff)
        elif op[0] == 'truncate':
            chain.truncate(chi, kappa, max_err, noisy)
        last = op[0]
    if noisy and last not in (None, 'truncate'):
        chain.kappa_truncate(kappa, max_err)
    return chain
