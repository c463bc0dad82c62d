"""Bond and Kraus-leg truncation of an evolved state (reference:
MPDOSimulator/TNNOptimizer.py).

The functions take the ``stateNodes`` that ``TensorCircuit.evolve`` hands
out and act on the GPU chain behind them, in place, as the reference's act
on its node list.  The engine runs the reference's QR left-to-right and SVD
right-to-left sweeps as one operation (``bondTruncate``) and the kappa pass
as another (``svdKappa_left2right``); the three sweeps are also offered one
at a time (``qr_left2right``, ``svd_right2left``, ``svd_left2right``).  Each
needs a connected chain, as the reference's do (they look up the shared
bond edges).
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


def qr_left2right(_qubits: List[QubitNode]):
    """TNNOptimizer.py:87-108: reduced QR of every site but the last over
    (left bond, physical, Kraus) x (right bond), R absorbed into the next
    site.  Changes the gauge only."""
    _chain(_qubits, 'qr_left2right').qr_left2right()


def svd_right2left(_qubits: List[QubitNode], max_singular_values: Optional[int] = None,
                   max_truncation_err: Optional[float] = None):
    """TNNOptimizer.py:111-134: for idx = n-1 .. 1, split the contracted pair
    (idx-1, idx) keeping at most ``max_singular_values`` (and the relative
    error rule), sqrt(S) on both sides.  Returns the discarded weight per
    bond (the reference drops it)."""
    return _chain(_qubits, 'svd_right2left').svd_sweep('right2left', max_singular_values, max_truncation_err)


def svd_left2right(_qubits: List[QubitNode], max_singular_values: int,
                   max_truncation_err: Optional[float] = None):
    """TNNOptimizer.py:137-161: the same split over the pairs (idx, idx+1) for
    idx = 0 .. n-2."""
    return _chain(_qubits, 'svd_left2right').svd_sweep('left2right', max_singular_values, max_truncation_err)


def cal_entropy(qubits):
    """TNNOptimizer.py:200-211 (not implemented in the reference either)."""
    raise NotImplementedError
