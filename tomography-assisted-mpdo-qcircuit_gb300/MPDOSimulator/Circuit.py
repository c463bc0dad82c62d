"""TensorCircuit: the reference's MPDO simulator API over the GB300 engine
(reference: MPDOSimulator/Circuit.py).

``evolve`` walks the queued layers exactly as the reference does
(Circuit.py:469-491): gates are contracted into the MPDO sites, ``truncate()``
layers run the QR left-to-right / SVD right-to-left bond sweep and then the
kappa SVD pass (only once the chain is connected), and a final kappa pass
follows when the last layer is not a truncate.  Every contraction and
factorisation runs on the GPU through ``libmpdo_gb300.so``; there is no CPU
path.
"""
from typing import Any, Dict, List, Optional, Union

import numpy as np
import torch

from .AbstractCircuit import QuantumCircuit
from .NoiseChannel import NoiseChannel
from .QuantumGates.AbstractGate import QuantumGate
from .QuantumGates.SingleGates import MeasureX, MeasureY
from .Tools import QubitNode, count_item
from . import dmOperations

GLOBAL_MINIMUM = 2.718281828459045 * 1e-8       # Circuit.py:22
MAX_ATTEMPTS = 4                                 # Circuit.py:23


def _cuda_index(device) -> int:
    if isinstance(device, int):
        return device
    if isinstance(device, str) and device.startswith('cuda'):
        return int(device.split(':')[1]) if ':' in device else 0
    return 0


class TensorCircuit(QuantumCircuit):
    def __init__(self, qn: int, ideal: bool = True, noiseType: str = 'no',
                 chiFileDict: Optional[Dict[str, Dict[str, Any]]] = None,
                 chi: Optional[int] = None, kappa: Optional[int] = None,
                 max_truncation_err: Optional[float] = None, chip: Optional[str] = None,
                 dtype=torch.complex64, device: Optional[Union[str, int]] = None):
        """Circuit.py:27-63.  ``device`` selects where returned tensors live; the
        evolution itself always runs on a CUDA device (``cuda:k`` picks which)."""
        super().__init__(noiseFiles=chiFileDict, chi=chi, kappa=kappa, max_truncation_err=max_truncation_err,
                         dtype=dtype, device=device)
        if dtype not in (torch.complex64, torch.complex128):
            raise ValueError('dtype must be torch.complex64 or torch.complex128')
        self.qnumber = qn
        self.ideal = ideal
        self.noiseType = noiseType.lower()
        self.Noise = None
        self._chain = None
        self.discarded_weights: List[np.ndarray] = []
        if not ideal:
            if self.noiseType not in ['unified', 'realnoise', 'idealnoise']:
                raise ValueError(f'Unsupported noise type: {self.noiseType}')
            self.Noise = NoiseChannel(chip=chip, dtype=dtype, device=self.device)
            self.unified = self.noiseType == 'unified'
            self.realNoise = self.noiseType == 'realnoise'
            self.idealNoise = self.noiseType == 'idealnoise'
            if self.realNoise:
                self._load_exp_tensors()

    # ---------------------------------------------------------- engine ---
    def _engine(self):
        from mpdo_gb300 import Engine
        return Engine.get(_cuda_index(self.device))

    @staticmethod
    def _np(t) -> np.ndarray:
        return t.detach().to('cpu', torch.complex128).numpy()

    @staticmethod
    def _gate_np(gate: QuantumGate) -> np.ndarray:
        f = getattr(gate, 'numpy_tensor', None)
        return f() if f is not None else gate.tensor.detach().to('cpu', torch.complex128).numpy()

    def _noisy_1q(self, gate: QuantumGate) -> np.ndarray:
        """Circuit.py:141-155 (composite cached per name for fixed gates)."""
        g = self._gate_np(gate)
        if not ((self.idealNoise or self.unified) and not gate.ideal):
            return g
        key = None if (gate.variational or gate.name == 'ArbSingleGate') else gate.name
        if key is not None and key in self.noiseTensorDict:
            return self.noiseTensorDict[key]
        # einsum('nlm, ljk, ji -> nimk', decay, dephasing, G): the gate-free
        # part is contracted once per pair of noise tensors
        pre_key = (id(self.Noise.decayTensor), id(self.Noise.dephasingTensor))
        if getattr(self, '_noise_pre_key', None) != pre_key:
            self._noise_pre = np.einsum('nlm,ljk->njmk', self._np(self.Noise.decayTensor),
                                        self._np(self.Noise.dephasingTensor))
            self._noise_pre_key = pre_key
        t = np.einsum('njmk,ji->nimk', self._noise_pre, g).reshape(2, 2, -1)
        if key is not None:
            self.noiseTensorDict[key] = t
        return t

    def _noisy_2q(self, gate: QuantumGate) -> np.ndarray:
        """Circuit.py:84-100: idealNoise appends 2q depolarising after the gate;
        realNoise gates (CZEXP/CPEXP) carry their own Kraus leg."""
        gnoise = (self.idealNoise and not gate.ideal) or self.realNoise
        if not gnoise or self.realNoise:
            return self._gate_np(gate)
        key = None if gate.variational else '2q:' + gate.name
        if key is not None and key in self.noiseTensorDict:
            return self.noiseTensorDict[key]
        # einsum('ijklp, klmn -> ijmnp', dpCTensor2, G) on the host: the
        # composite is a 16 x 16 x K product, smaller than a device round trip
        dkey = id(self.Noise.dpCTensor2)
        if getattr(self, '_dpc2_key', None) != dkey:
            self._dpc2 = self._np(self.Noise.dpCTensor2)
            self._dpc2_key = dkey
        t = np.einsum('ijklp,klmn->ijmnp', self._dpc2, self._gate_np(gate).reshape(2, 2, 2, 2))
        if key is not None:
            self.noiseTensorDict[key] = t
        return t

    def _gate_ops(self, _layer_num: int, _oqs: List[int], _gate: Optional[QuantumGate] = None) -> list:
        """Circuit.py:180-224: the engine operations of one gate layer,
        ('1q', site, kraus[2,2,K]) per target or ('2q', site_min,
        kraus[o_min,o_max,i_min,i_max,K])."""
        if not isinstance(_oqs, list):
            raise TypeError('Operating qubits must be a list.')
        if _oqs[0] is None:
            return []
        if max(_oqs) >= self.qnumber:
            raise ValueError(f'Qubit index out of range, max index is Q{max(_oqs)}.')
        gate = _gate or self.layers[_layer_num]
        if not gate or gate.name == 'MeasureZ':
            return []
        if not isinstance(gate, QuantumGate):
            raise TypeError(f'Gate must be a QuantumGate, current type is {type(gate)}.')
        if gate.single:
            t = self._noisy_1q(gate)
            return [('1q', q, t) for q in _oqs]
        if len(_oqs) != 2 or _oqs[0] == _oqs[1]:
            raise ValueError('Invalid operating qubits for a two-qubit gate.')
        a, b = _oqs
        if abs(a - b) != 1:
            raise ValueError('Only nearest-neighbour two-qubit gates are supported by the MPDO engine.')
        t = self._noisy_2q(gate)
        if t.ndim == 4:
            t = t[..., None]
        if a > b:
            t = np.transpose(t, (1, 0, 3, 2, 4))
        return [('2q', min(a, b), t)]

    def _add_gate(self, chain, _layer_num: int, _oqs: List[int], _gate: Optional[QuantumGate] = None):
        """Circuit.py:180-224."""
        for op in self._gate_ops(_layer_num, _oqs, _gate):
            if op[0] == '1q':
                chain.apply_1q(op[1], op[2])
            else:
                chain.apply_2q(op[1], op[2], GLOBAL_MINIMUM)

    def _engine_ops(self) -> list:
        """Every engine operation evolve() performs, in order (Circuit.py:469-491):
        gate ops, ('truncate',) per truncate layer and a final ('kappa',) when
        the last layer of a noisy circuit is not a truncate."""
        ops, last = [], None
        for i, layer in enumerate(self.layers):
            name = layer.name.lower()
            if 'truncate' in name:
                ops.append(('truncate',))
            elif 'barrier' not in name:
                ops += self._gate_ops(i, self._oqs_list[i], layer)
            last = name
        if not self.ideal and last is not None and 'truncate' not in last:          # Circuit.py:487-489
            ops.append(('kappa',))
        return ops

    def _initial(self, state: List[QubitNode]):
        if len(state) != self.qnumber:
            raise ValueError('state length differs from the number of qubits')
        self._initState = [QubitNode(s.tensor.clone(), s.name, s.axis_names, s.connected) for s in state]
        vectors = np.stack([self._np(s.tensor).reshape(2) for s in state])
        connected = all(getattr(s, 'connected', False) for s in state)
        dt = 'complex128' if self.dtype == torch.complex128 else 'complex64'
        return vectors, connected, dt

    def _attach_chain(self, chain, state: List[QubitNode]):
        self._chain = chain
        self._dm, self._dmNodes, self._vector = None, None, None
        nodes = [QubitNode(None, f'qubit_{k}', [f'bond_{k - 1}_{k}', f'physics_{k}', f'I_{k}', f'bond_{k}_{k + 1}'],
                           chain=chain, index=k, dtype=self.dtype, device=self.device) for k in range(self.qnumber)]
        self._stateNodes = nodes
        state[:] = nodes
        return nodes

    def evolve(self, state: List[QubitNode]):
        """Circuit.py:469-491."""
        from mpdo_gb300 import Chain
        vectors, connected, dt = self._initial(state)
        ops = self._engine_ops()
        chain = Chain(vectors, dtype=dt, connected=connected, engine=self._engine())
        noisy = not self.ideal
        self.discarded_weights = []
        for op in ops:
            if op[0] == '1q':
                chain.apply_1q(op[1], op[2])
            elif op[0] == '2q':
                chain.apply_2q(op[1], op[2], GLOBAL_MINIMUM)
            elif op[0] == 'truncate':
                self.discarded_weights.append(
                    chain.truncate(self.chi, self.kappa, self.max_truncation_err, noisy, report=True))
            else:
                chain.kappa_truncate(self.kappa, self.max_truncation_err)
        return self._attach_chain(chain, state)

    def forward(self, state):
        self.evolve(state)

    def _need_chain(self):
        if self._chain is None:
            raise RuntimeError('evolve(state) first')
        return self._chain

    # --------------------------------------------------------- readout ---
    def cal_vector(self):
        """Circuit.py:264-272 (ideal circuits only)."""
        if not self.ideal:
            raise ValueError('Noisy circuit cannot be represented by state vector efficiently.')
        ch = self._need_chain()
        psi = np.ones((1, 1), dtype=np.complex128)
        for k in range(self.qnumber):
            a = ch.site(k)                                        # (l, 2, 1, r)
            psi = np.einsum('pl,lsr->psr', psi, a[:, :, 0, :]).reshape(-1, a.shape[3])
        v = torch.as_tensor(psi.reshape(2 ** self.qnumber, 1)).to(dtype=self.dtype, device=self.device)
        self._vector = v
        return v

    def cal_dmNodes(self, reduced_index: Optional[List] = None):
        """Circuit.py:274-280: a handle on the doubled network (ket + conj)."""
        nodes = dmOperations.DMNodes(self._need_chain(), self.qnumber, self.dtype, self.device)
        if reduced_index:
            nodes.trace_out(reduced_index)
        self._dmNodes = nodes
        return nodes

    def cal_dm(self, reduced_index: Optional[List] = None, _replicate_require: bool = False):
        """Circuit.py:282-295: rho (or the reduced rho with ``reduced_index``
        traced out), rows = ket legs, qubit order ascending."""
        reduced_index = [] if reduced_index is None else list(reduced_index)
        if reduced_index and max(reduced_index) >= self.qnumber:
            raise ValueError('Reduced index should not be larger than the qubit number.')
        keep = [q for q in range(self.qnumber) if q not in reduced_index]
        rho = self._need_chain().reduced_dm(keep)
        self._dm = torch.as_tensor(rho).to(dtype=self.dtype, device=self.device)
        return self._dm

    def probabilities(self, keep: Optional[List[int]] = None) -> torch.Tensor:
        """Diagonal of the (reduced) density matrix without forming it."""
        p = self._need_chain().probs(keep)
        return torch.as_tensor(p)

    # -------------------------------------------------------- sampling ---
    def _sample_source(self, nodes):
        """The chain behind ``nodes`` (Circuit.py:412-413 replicates the given
        nodes, else the circuit's own state)."""
        if nodes is None:
            return self._need_chain()
        chains = [getattr(n, '_chain', None) for n in nodes]
        if len(chains) != self.qnumber or chains[0] is None or any(c is not chains[0] for c in chains):
            raise ValueError('_stateNodes4Sample must be the stateNodes of one evolved state of '
                             f'{self.qnumber} qubits')
        return chains[0]

    def _conditional_prb(self, chain, order: List[int], history: List[int]) -> float:
        """Circuit.py:297-332: p(1 | history) on qubit order[len(history)],
        the other unmeasured qubits traced, GLOBAL_MINIMUM added to both."""
        q = order[len(history)]
        proj = [np.diag([1.0, 0.0]).astype(np.complex128), np.diag([0.0, 1.0]).astype(np.complex128)]
        ops = {order[j]: proj[h] for j, h in enumerate(history)}
        p = []
        for v in (0, 1):
            o = dict(ops)
            o[q] = proj[v]
            p.append(chain.expect_ops(o) + GLOBAL_MINIMUM)
        p = np.asarray(p)
        if (p < 0).any():
            raise RuntimeError(f'State is illegal, and your probability distribution is {p}.')
        return float(p[1] / p.sum())

    def sample(self, shots: Optional[int] = None, orientation: Optional[List[int]] = None,
               reduced: Optional[List[int]] = None, sample_string: bool = True, _tqdm_disable: bool = False,
               _require_sequential_sample: bool = False, _require_bool_result: bool = False,
               _require_counts: bool = True, _stateNodes4Sample=None):
        """Circuit.py:389-446 (batch conditional sampling, 344-387): shots
        sharing a measured prefix form one group; each group's conditional
        probability p(1 | prefix) (GLOBAL_MINIMUM added to both outcomes)
        splits it binomially.  ``_require_sequential_sample`` (the reference's
        one-shot-at-a-time loop, Circuit.py:334-342) draws from the same
        distribution, so both run the grouped sampler.  ``_stateNodes4Sample``
        samples another evolved state (the ``stateNodes`` of a circuit)."""
        shots = shots or 1024
        reduced = reduced or []
        order = [q for q in range(self.qnumber) if q not in reduced]
        L = len(order)
        orientation = orientation or [2] * L
        if len(orientation) != L:
            raise ValueError('Length of orientation must match the sample length. Check reduced or unmeasured qubits.')
        chain = self._sample_source(_stateNodes4Sample).clone()
        if not _tqdm_disable:
            print(f'Sample Direction:\n (scheme-{"".join("XYZ"[v] for v in orientation)})')
        for val, M in [(0, MeasureX), (1, MeasureY)]:
            idx = [order[i] for i, v in enumerate(orientation) if v == val]
            if idx:
                g = self._np(M(dtype=self.dtype, device='cpu').tensor)
                for q in idx:
                    chain.apply_1q(q, g)
        # conditional sampling on the GPU (right environments cached, all
        # groups of a prefix advanced together); the binomial splits draw
        # from a seed taken from torch's generator, so torch.manual_seed
        # makes runs reproducible
        seed = int(torch.randint(0, 2 ** 62, (1,)).item())
        raw = chain.sample(order, shots, seed, GLOBAL_MINIMUM)
        seq = torch.from_numpy(raw.astype(np.bool_ if _require_bool_result else np.int32))
        bits = seq.tolist()
        if sample_string and not _require_bool_result:
            bits = [''.join(map(str, b)) for b in bits]
        self._samples = bits
        if _require_counts:
            self._counts = count_item(bits)
            return self._samples, self._counts
        return self._samples

    def randomSample(self, measurement_schemes: List[List[int]], shots_per_scheme: int = 1024,
                     reduced: Optional[List[int]] = None, _tqdm_disable: bool = False,
                     _require_sequential_sample: bool = False, _require_bool_result: bool = False,
                     _stateNodes4Sample=None):
        """Circuit.py:448-466: ``shots_per_scheme`` samples in each scheme
        (per measured qubit 0 = X, 1 = Y, 2 = Z), as a list over schemes of
        bit lists.  All schemes run in one engine call that builds the right
        environments once; scheme s draws from the seed a ``sample`` call
        would take at its turn, so the result equals the reference's loop of
        ``sample`` calls under the same ``torch.manual_seed``."""
        reduced = reduced or []
        order = [q for q in range(self.qnumber) if q not in reduced]
        L = len(order)
        schemes = [list(s) for s in measurement_schemes]
        for s in schemes:
            if len(s) != L:
                raise ValueError('Length of orientation must match the sample length. Check reduced or unmeasured '
                                 'qubits.')
        if not schemes:
            return []
        chain = self._sample_source(_stateNodes4Sample)
        rot = np.stack([self._np(M(dtype=self.dtype, device='cpu').tensor) for M in (MeasureX, MeasureY)])
        seeds = [int(torch.randint(0, 2 ** 62, (1,)).item()) for _ in schemes]
        raw = chain.sample_schemes(order, schemes, shots_per_scheme, seeds, rot, GLOBAL_MINIMUM)
        return [torch.from_numpy(r.astype(np.bool_ if _require_bool_result else np.int32)).tolist() for r in raw]


def evolve_batch(circuits: List[TensorCircuit], states: Optional[List[List[QubitNode]]] = None,
                 workers: int = 16) -> List[dict]:
    """Evolve many independent circuits concurrently on one GPU (no
    counterpart in the reference, whose callers loop over ``evolve``).

    Each circuit ends exactly as after its own ``evolve(state)``: the same
    engine operations run on one of ``workers`` engines (own stream and memory
    pool each), and the circuit's state, ``discarded_weights`` and readouts
    are attached to it.  ``states`` defaults to |0...0> for every circuit.
    Returns per circuit dict(z=<Z_i>, zz=<Z_i Z_{i+1}>, discarded=per-bond
    weights of every truncate layer), computed by the worker right after the
    evolution (not normalised by Tr rho, as ``dmOperations.pauli_expect``)."""
    from mpdo_gb300 import Batch
    from .Tools import create_ket0Series
    if not circuits:
        return []
    devs = {_cuda_index(c.device) for c in circuits}
    if len(devs) != 1:
        raise ValueError('all circuits of a batch must select the same CUDA device')
    if states is None:
        states = [create_ket0Series(c.qnumber, dtype=c.dtype) for c in circuits]
    if len(states) != len(circuits):
        raise ValueError('one initial state per circuit')
    progs = []
    for c, st in zip(circuits, states):
        vectors, connected, dt = c._initial(st)
        progs.append(dict(n=c.qnumber, dtype=dt, vectors=vectors, connected=connected, chi=c.chi, kappa=c.kappa,
                          max_err=c.max_truncation_err, noisy=not c.ideal, cutoff=GLOBAL_MINIMUM,
                          ops=c._engine_ops(), z=True, zz=True, discarded=True))
    results = Batch.get(devs.pop(), workers).run(progs, keep_chains=True)
    for c, st, r in zip(circuits, states, results):
        c.discarded_weights = [row.copy() for row in r['discarded']]
        c._attach_chain(r.pop('chain'), st)
    return results
