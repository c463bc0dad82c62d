"""Bond and Kraus-leg truncation of an evolved state (reference:
MPDOSimulator/TNNOptimizer.py).

The functions take the ``stateNodes`` that ``TensorCircuit.evolve`` hands
out and act on the GPU chain behind them, in place, as the reference's act
on its node list.  The engine runs the reference's QR left-to-right and SVD
right-to-left sweeps as one operation (``bondTruncate``) and the kappa pass
as another (``svdKappa_left2right``).  The sweeps are not offered one at a
time: ``qr_left2right`` alone only changes the gauge, and the evolution
never calls ``svd_right2left`` or ``svd_left2right`` on their own.
"""
from typing import List, Optional

from .Tools import QubitNode


def _validate_qubit_list(qubits, func_name: str):
    """TNNOptimizer.py:64-69."""
    if not isinstance(qubits, list):
        raise TypeError(f'`{func_name}` expects a list of qubit nodes, got {type(qubits).__name__}')


def _chain(qubits: List[QubitNode], func_name: str):
    _validate_qubit_list(qubits, func_name)
    chains = [getattr(q, '_chain', None) for q in qubits]
    ch = chains[0] if chains else None
    if ch is None or any(c is not ch for c in chains) or len(qubits) != ch.n:
        raise ValueError(f'`{func_name}` expects the stateNodes of one evolved state (TensorCircuit.evolve)')
    return ch


def checkConnectivity(_qubits: List[QubitNode]) -> bool:
    """TNNOptimizer.py:51-61: every neighbouring pair shares a bond.  Product
    states from ``Tools.create_ket*Series`` are connected only when created
    with ``connected=True``."""
    if len(_qubits) <= 1:
        return True
    if all(getattr(q, '_chain', None) is None for q in _qubits):
        return all(getattr(q, 'connected', False) for q in _qubits)
    ch = _chain(_qubits, 'checkConnectivity')
    return all(ch.bond_present(b) for b in range(ch.n - 1))


def bondTruncate(_qubits: List[QubitNode], max_singular_values: Optional[int] = None,
                 max_truncation_err: Optional[float] = None, regularization: bool = False):
    """TNNOptimizer.py:72-84: QR left-to-right then SVD right-to-left keeping
    at most ``max_singular_values`` per bond (and the relative error rule).
    ``regularization`` without a cap only re-gauges the chain, which leaves
    every readout unchanged, so it does nothing here.  A chain that is not
    connected is left as it is (the engine truncates connected chains only,
    the condition evolve() checks first, Circuit.py:477)."""
    if max_singular_values is None and max_truncation_err is None:
        return None
    _chain(_qubits, 'bondTruncate').truncate(max_singular_values, None, max_truncation_err, False)


def svdKappa_left2right(_qubits: List[QubitNode], max_singular_values: Optional[int] = None,
                        max_truncation_err: Optional[float] = None):
    """TNNOptimizer.py:164-197: per site whose Kraus leg is wider than
    ``max_singular_values``, an SVD keeping that many (and the relative error
    rule); the site becomes U.S."""
    if max_singular_values is None and max_truncation_err is None:
        return None
    _chain(_qubits, 'svdKappa_left2right').kappa_truncate(max_singular_values, max_truncation_err)


def _single_sweep(name: str):
    def f(*args, **kwargs):
        raise NotImplementedError(f'`{name}` alone is not offered by the GB300 engine: bondTruncate runs the '
                                  'QR left-to-right and SVD right-to-left sweeps as one operation')
    f.__name__ = name
    f.__doc__ = f'TNNOptimizer.py `{name}`: not offered on its own (see bondTruncate).'
    return f


qr_left2right = _single_sweep('qr_left2right')
svd_right2left = _single_sweep('svd_right2left')
svd_left2right = _single_sweep('svd_left2right')


def cal_entropy(qubits):
    """TNNOptimizer.py:200-211 (not implemented in the reference either)."""
    raise NotImplementedError
