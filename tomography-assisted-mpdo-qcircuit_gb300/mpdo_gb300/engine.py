"""Python handle over the C ABI: one ``Engine`` per device, ``Chain`` objects
holding an MPDO on that device.  Arrays cross the boundary as host numpy
buffers (complex values as interleaved float64)."""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check, load

_engines: Dict[int, 'Engine'] = {}


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _cplx(a) -> np.ndarray:
    """complex array -> contiguous interleaved float64 view."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    return a.view(np.float64)


class Engine:
    def __init__(self, device: int = 0):
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.mpdo_engine_create(int(device), C.byref(h)))
        self.handle = h
        self.device = int(device)

    @classmethod
    def get(cls, device: int = 0) -> 'Engine':
        if device not in _engines:
            _engines[device] = cls(device)
        return _engines[device]

    def set_option(self, name: str, value: float) -> None:
        check(self._lib.mpdo_engine_set_option(self.handle, name.encode(), float(value)))

    def sync(self) -> None:
        check(self._lib.mpdo_engine_sync(self.handle))

    def set_stream(self, stream_ptr: Optional[int]) -> None:
        check(self._lib.mpdo_engine_set_stream(self.handle, C.c_void_p(stream_ptr or 0)))

    def debug_qr(self, a, dtype: str = 'complex128'):
        """Kernel test hook: Householder QR of a host matrix on the GPU."""
        a = np.asarray(a, dtype=np.complex128)
        m, n = a.shape
        k = min(m, n)
        q = np.zeros(2 * m * k)
        r = np.zeros(2 * k * n)
        check(self._lib.mpdo_debug_qr(self.handle, _lib.MPDO_C128 if dtype.endswith('128') else _lib.MPDO_C64,
                                      m, n, _dptr(_cplx(a)), _dptr(q), _dptr(r)))
        return q.view(np.complex128).reshape(m, k), r.view(np.complex128).reshape(k, n)

    def debug_svd(self, a, dtype: str = 'complex128'):
        """Kernel test hook: right singular vectors (QR + one-sided Jacobi)."""
        a = np.asarray(a, dtype=np.complex128)
        m, n = a.shape
        w = np.zeros(2 * n * n)
        s = np.zeros(n)
        check(self._lib.mpdo_debug_svd(self.handle, _lib.MPDO_C128 if dtype.endswith('128') else _lib.MPDO_C64,
                                       m, n, _dptr(_cplx(a)), _dptr(w), _dptr(s)))
        return w.view(np.complex128).reshape(n, n).T, s

    def debug_split(self, y, keep: int, dtype: str = 'complex128'):
        """Kernel test hook: Y ~= L R with L = U sqrt(S), R = sqrt(S) V^H (top keep)."""
        y = np.asarray(y, dtype=np.complex128)
        m, n = y.shape
        lo = np.zeros(2 * m * keep)
        ro = np.zeros(2 * keep * n)
        check(self._lib.mpdo_debug_split(self.handle, _lib.MPDO_C128 if dtype.endswith('128') else _lib.MPDO_C64,
                                         m, n, int(keep), _dptr(_cplx(y)), _dptr(lo), _dptr(ro)))
        return lo.view(np.complex128).reshape(m, keep), ro.view(np.complex128).reshape(keep, n)

    KERNEL_CLASSES = ('gemm', 'qr_factor', 'qr_apply', 'jacobi', 'kraus1q', 'mix2q', 'other', None, 'bjacobi',
                      None, None, None, None, 'hetrd')
    PHASES = ('qr_sweep', 'svd_sweep', 'kappa_pass', 'wide_svd')

    def profile(self, enable: bool) -> None:
        check(self._lib.mpdo_engine_profile(self.handle, int(bool(enable))))

    def profile_read(self) -> dict:
        """{class: dict(launches, ms, flops, bytes)} accumulated since profile(True),
        plus 'wide_bonds' (range finder / exact counts) and 'phases' ({phase:
        dict(count, ms)} for the QR sweep, SVD sweep, kappa pass and the
        wide-bond SVDs inside the SVD sweep)."""
        out = {}
        for i, name in enumerate(self.KERNEL_CLASSES):
            if name is None:
                continue
            n, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
            check(self._lib.mpdo_engine_profile_read(self.handle, i, C.byref(n), C.byref(ms), C.byref(fl), C.byref(by)))
            out[name] = dict(launches=int(n.value), ms=ms.value, flops=fl.value, bytes=by.value)
        n, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        check(self._lib.mpdo_engine_profile_read(self.handle, 7, C.byref(n), C.byref(ms), C.byref(fl), C.byref(by)))
        out['wide_bonds'] = dict(range_finder=int(n.value), exact=int(fl.value), max_residual=by.value,
                                 tridiagonal=int(ms.value))
        phases = {}
        for i, name in enumerate(self.PHASES, start=9):
            n, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
            check(self._lib.mpdo_engine_profile_read(self.handle, i, C.byref(n), C.byref(ms), C.byref(fl), C.byref(by)))
            phases[name] = dict(count=int(n.value), ms=ms.value)
        out['phases'] = phases
        return out

    def launch_histogram(self) -> Dict[str, int]:
        """Kernel launches so far per launcher function (all engines)."""
        buf = C.create_string_buffer(1 << 16)
        check(self._lib.mpdo_launch_histogram(buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt = line.rsplit(' ', 1)
            out[name] = int(cnt)
        return out

    def launch_count(self) -> int:
        c = C.c_uint64()
        check(self._lib.mpdo_engine_launch_count(self.handle, C.byref(c)))
        return int(c.value)


class Chain:
    """An MPDO on the GPU (site tensors A[l][s][a][r])."""

    def __init__(self, vectors, dtype: str = 'complex64', connected: bool = False,
                 engine: Optional[Engine] = None, _handle=None):
        self.engine = engine or Engine.get(0)
        self._lib = self.engine._lib
        self.dtype = 'complex128' if str(dtype).endswith('128') else 'complex64'
        if _handle is not None:
            self.handle = _handle
        else:
            v = _cplx(np.asarray(vectors, dtype=np.complex128).reshape(-1, 2))
            h = C.c_void_p()
            check(self._lib.mpdo_chain_create(self.engine.handle, v.size // 4,
                                              _lib.MPDO_C128 if self.dtype == 'complex128' else _lib.MPDO_C64,
                                              _dptr(v), int(bool(connected)), C.byref(h)))
            self.handle = h
        n = C.c_int()
        check(self._lib.mpdo_chain_num_sites(self.handle, C.byref(n)))
        self.n = n.value

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            try:
                self._lib.mpdo_chain_destroy(h)
            except Exception:
                pass
            self.handle = None

    def clone(self) -> 'Chain':
        h = C.c_void_p()
        check(self._lib.mpdo_chain_clone(self.handle, C.byref(h)))
        return Chain(None, self.dtype, engine=self.engine, _handle=h)

    # ---- gates ------------------------------------------------------------
    def apply_1q(self, site: int, kraus) -> None:
        k = np.asarray(kraus, dtype=np.complex128)
        if k.ndim == 2:
            k = k[:, :, None]
        buf = _cplx(k)
        check(self._lib.mpdo_apply_1q(self.handle, int(site), _dptr(buf), int(k.shape[-1])))

    def apply_2q(self, site_min: int, kraus, cutoff: float) -> None:
        k = np.asarray(kraus, dtype=np.complex128)
        if k.ndim == 4:
            k = k[..., None]
        buf = _cplx(k)
        check(self._lib.mpdo_apply_2q(self.handle, int(site_min), _dptr(buf), int(k.shape[-1]), float(cutoff)))

    def truncate(self, chi: Optional[int], kappa: Optional[int], max_err: Optional[float], noisy: bool,
                 report: bool = False):
        out = np.zeros(max(self.n - 1, 1), dtype=np.float64) if report else None
        check(self._lib.mpdo_truncate(self.handle, int(chi or 0), int(kappa or 0),
                                      -1.0 if max_err is None else float(max_err), int(bool(noisy)),
                                      _dptr(out) if report else None))
        return out[: self.n - 1] if report else None

    def sample(self, order: Sequence[int], shots: int, seed: int, pfloor: float = 2.718281828459045e-8) -> np.ndarray:
        """Conditional sampling of the ascending qubits ``order`` (others
        traced): shots x len(order) array of 0/1 (int8)."""
        o = np.ascontiguousarray(np.asarray(order, dtype=np.int32))
        out = np.zeros((int(shots), len(o)), dtype=np.int8)
        check(self._lib.mpdo_sample(self.handle, o.ctypes.data_as(C.POINTER(C.c_int)), len(o), int(shots),
                                    int(seed) & (2 ** 64 - 1), float(pfloor),
                                    out.ctypes.data_as(C.POINTER(C.c_int8))))
        return out

    def sample_schemes(self, order: Sequence[int], schemes, shots: int, seeds: Sequence[int], rot=None,
                       pfloor: float = 2.718281828459045e-8) -> np.ndarray:
        """Conditional sampling in several measurement schemes at once
        (``schemes``: S x len(order) of 0 = X, 1 = Y, 2 = Z; ``rot``: the X
        and Y basis-change gates, 2 x 2 x 2 complex): S x shots x len(order)
        array of 0/1 (int8).  Scheme s equals ``sample`` with ``seeds[s]`` on
        a copy rotated by those gates."""
        o = np.ascontiguousarray(np.asarray(order, dtype=np.int32))
        sc = np.ascontiguousarray(np.asarray(schemes, dtype=np.int32).reshape(-1, len(o)))
        S = sc.shape[0]
        sd = np.ascontiguousarray(np.asarray([int(x) & (2 ** 64 - 1) for x in seeds], dtype=np.uint64))
        if sd.size != S:
            raise ValueError('one seed per scheme')
        rb = None if rot is None else _cplx(np.asarray(rot, dtype=np.complex128).reshape(2, 2, 2))
        out = np.zeros((S, int(shots), len(o)), dtype=np.int8)
        check(self._lib.mpdo_sample_schemes(self.handle, o.ctypes.data_as(C.POINTER(C.c_int)), len(o),
                                            sc.ctypes.data_as(C.POINTER(C.c_int)), S, int(shots),
                                            sd.ctypes.data_as(C.POINTER(C.c_uint64)), float(pfloor),
                                            None if rb is None else _dptr(rb),
                                            out.ctypes.data_as(C.POINTER(C.c_int8))))
        return out

    def qr_left2right(self) -> None:
        """TNNOptimizer.py:87-108 on its own."""
        check(self._lib.mpdo_qr_left2right(self.handle))

    def svd_sweep(self, direction: str, chi: Optional[int], max_err: Optional[float]) -> np.ndarray:
        """TNNOptimizer.py:111-161: 'right2left' or 'left2right' SVD sweep on
        its own; returns the per-bond discarded weight."""
        out = np.zeros(max(self.n - 1, 1), dtype=np.float64)
        fn = self._lib.mpdo_svd_right2left if direction == 'right2left' else self._lib.mpdo_svd_left2right
        check(fn(self.handle, int(chi or 0), -1.0 if max_err is None else float(max_err), _dptr(out)))
        return out[: self.n - 1]

    def kappa_truncate(self, kappa: Optional[int], max_err: Optional[float]) -> None:
        check(self._lib.mpdo_kappa_truncate(self.handle, int(kappa or 0),
                                            -1.0 if max_err is None else float(max_err)))

    # ---- inspection -------------------------------------------------------
    def site_dims(self, site: int):
        d = (C.c_int * 4)()
        check(self._lib.mpdo_chain_site_dims(self.handle, int(site), d))
        return tuple(d)

    def dims(self):
        return [self.site_dims(i) for i in range(self.n)]

    def bond_present(self, bond: int) -> bool:
        p = C.c_int()
        check(self._lib.mpdo_chain_bond_present(self.handle, int(bond), C.byref(p)))
        return bool(p.value)

    def site(self, i: int) -> np.ndarray:
        d = self.site_dims(i)
        out = np.zeros(int(np.prod(d)) * 2, dtype=np.float64)
        check(self._lib.mpdo_chain_read_site(self.handle, int(i), _dptr(out)))
        return out.view(np.complex128).reshape(d)

    def write_site(self, i: int, tensor) -> None:
        t = np.asarray(tensor, dtype=np.complex128)
        d = (C.c_int * 4)(*t.shape)
        buf = _cplx(t)
        check(self._lib.mpdo_chain_write_site(self.handle, int(i), d, _dptr(buf)))

    def _torch_dtype(self):
        import torch
        return torch.complex64 if self.dtype == 'complex64' else torch.complex128

    def site_tensor(self, i: int):
        """Site i as a torch tensor (l, 2, a, r) on the engine's device, in the
        chain's precision, copied device to device (``mpdo_chain_read_site_device``)."""
        import torch
        out = torch.empty(self.site_dims(i), dtype=self._torch_dtype(), device=f'cuda:{self.engine.device}')
        check(self._lib.mpdo_chain_read_site_device(self.handle, int(i), C.c_void_p(out.data_ptr())))
        return out

    def write_site_tensor(self, i: int, tensor) -> None:
        """Replace site i by a torch tensor (l, 2, a, r) without a host copy: it is
        brought to the engine's device and the chain's precision, the work that
        produced it is waited for, and it is copied device to device
        (``mpdo_chain_write_site_device``)."""
        import torch
        t = tensor.to(device=f'cuda:{self.engine.device}', dtype=self._torch_dtype()).contiguous()
        if t.dim() != 4 or t.shape[1] != 2:
            raise ValueError(f'a site tensor has shape (l, 2, a, r), got {tuple(t.shape)}')
        torch.cuda.current_stream(t.device).synchronize()
        d = (C.c_int * 4)(*t.shape)
        check(self._lib.mpdo_chain_write_site_device(self.handle, int(i), d, C.c_void_p(t.data_ptr())))

    # ---- readout ----------------------------------------------------------
    def reduced_dm(self, keep: Optional[Sequence[int]] = None) -> np.ndarray:
        keep = list(range(self.n)) if keep is None else sorted(int(q) for q in keep)
        m = len(keep)
        arr = (C.c_int * max(m, 1))(*keep)
        out = np.zeros(2 * 4 ** m, dtype=np.float64)
        check(self._lib.mpdo_reduced_dm(self.handle, arr, m, _dptr(out)))
        return out.view(np.complex128).reshape(2 ** m, 2 ** m)

    def trace_rho_rho(self, other: Optional['Chain'] = None, keep: Optional[Sequence[int]] = None) -> float:
        """Re Tr(rho_self rho_other) with both states traced over the qubits
        not in ``keep`` (default: all kept), for any number of kept qubits."""
        other = self if other is None else other
        keep = list(range(self.n)) if keep is None else sorted(int(q) for q in keep)
        arr = (C.c_int * max(len(keep), 1))(*keep)
        out = C.c_double()
        check(self._lib.mpdo_trace_rho_rho(self.handle, other.handle, arr, len(keep), C.byref(out)))
        return out.value

    def probs(self, keep: Optional[Sequence[int]] = None) -> np.ndarray:
        keep = list(range(self.n)) if keep is None else sorted(int(q) for q in keep)
        m = len(keep)
        arr = (C.c_int * max(m, 1))(*keep)
        out = np.zeros(2 ** m, dtype=np.float64)
        check(self._lib.mpdo_probs(self.handle, arr, m, _dptr(out)))
        return out

    def expect_ops(self, ops: Dict[int, np.ndarray]) -> float:
        sites = sorted(ops)
        arr = (C.c_int * max(len(sites), 1))(*sites)
        buf = _cplx(np.stack([np.asarray(ops[q], dtype=np.complex128).reshape(2, 2) for q in sites])
                    if sites else np.zeros((1, 2, 2)))
        out = C.c_double()
        check(self._lib.mpdo_expect_ops(self.handle, arr, _dptr(buf), len(sites), C.byref(out)))
        return float(out.value)

    def expect_pauli_batch(self, codes) -> np.ndarray:
        codes = np.ascontiguousarray(np.asarray(codes, dtype=np.int8).reshape(-1, self.n))
        out = np.zeros(codes.shape[0], dtype=np.float64)
        check(self._lib.mpdo_expect_pauli_batch(self.handle, codes.ctypes.data_as(C.POINTER(C.c_int8)),
                                                codes.shape[0], _dptr(out)))
        return out


class Batch:
    """Independent circuits run concurrently (``mpdo_batch_*``): ``workers``
    host threads, each with its own engine (stream + memory pool) on one
    device, take whole circuits longest first.  ``run`` takes host programs
    and returns per-circuit readouts and, optionally, the final chains."""

    _cache: Dict[tuple, 'Batch'] = {}

    def __init__(self, device: int = 0, workers: int = 16):
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.mpdo_batch_create(int(device), int(workers), C.byref(h)))
        self.handle = h
        self.device = int(device)
        n = C.c_int()
        check(self._lib.mpdo_batch_num_workers(self.handle, C.byref(n)))
        self.workers = n.value
        self.engines = []
        for w in range(self.workers):
            eh = C.c_void_p()
            check(self._lib.mpdo_batch_engine(self.handle, w, C.byref(eh)))
            e = Engine.__new__(Engine)
            e._lib, e.handle, e.device, e._owner = self._lib, eh, self.device, self
            self.engines.append(e)

    @classmethod
    def get(cls, device: int = 0, workers: int = 16) -> 'Batch':
        key = (int(device), int(workers))
        if key not in cls._cache:
            cls._cache[key] = cls(device, workers)
        return cls._cache[key]

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            try:
                self._lib.mpdo_batch_destroy(h)
            except Exception:
                pass
            self.handle = None

    def set_option(self, name: str, value: float) -> None:
        check(self._lib.mpdo_batch_set_option(self.handle, name.encode(), float(value)))

    def run(self, programs: Sequence[dict], keep_chains: bool = False):
        """Each program: dict(n, dtype ('complex64'|'complex128'), vectors (n x 2),
        connected, chi, kappa, max_err, noisy, cutoff, ops, z, zz, discarded)
        with ops a list of ('1q', site, kraus[2,2,K]) / ('2q', site_min,
        kraus[o_min,o_max,i_min,i_max,K]) / ('truncate',) / ('kappa',).
        Returns one dict per program: z, zz, discarded (as requested) and
        chain (when keep_chains)."""
        kinds = {'1q': _lib.MPDO_OP_1Q, '2q': _lib.MPDO_OP_2Q, 'truncate': _lib.MPDO_OP_TRUNCATE,
                 'kappa': _lib.MPDO_OP_KAPPA}
        arr = (_lib.Program * max(1, len(programs)))()
        alive, outs = [], []
        for i, p in enumerate(programs):
            n = int(p['n'])
            ops = p['ops']
            kind = np.array([kinds[o[0]] for o in ops], dtype=np.int32)
            site = np.array([o[1] if len(o) > 1 else 0 for o in ops], dtype=np.int32)
            tens = [np.ascontiguousarray(np.asarray(o[2], dtype=np.complex128)) if len(o) > 2 else None for o in ops]
            kk = np.array([t.shape[-1] if t is not None and t.ndim in (3, 5) else 1 for t in tens], dtype=np.int32)
            sizes = [2 * t.size if t is not None else 0 for t in tens]
            off = np.zeros(len(ops), dtype=np.int64)
            if len(ops) > 1:
                off[1:] = np.cumsum(sizes[:-1])
            flat = np.concatenate([t.view(np.float64).ravel() for t in tens if t is not None]) \
                if any(t is not None for t in tens) else np.zeros(1)
            vec = _cplx(np.asarray(p['vectors'], dtype=np.complex128).reshape(n, 2))
            ntr = int(sum(1 for o in ops if o[0] == 'truncate'))
            o = {'z': np.zeros(n) if p.get('z') else None, 'zz': np.zeros(max(n - 1, 1)) if p.get('zz') else None,
                 'discarded': np.zeros(max(ntr * (n - 1), 1)) if p.get('discarded') else None}
            max_err = p.get('max_err')
            pr = arr[i]
            pr.n, pr.connected = n, int(bool(p.get('connected', False)))
            pr.dtype = _lib.MPDO_C128 if str(p.get('dtype', 'complex64')).endswith('128') else _lib.MPDO_C64
            pr.vectors = _dptr(vec)
            pr.chi, pr.kappa = int(p.get('chi') or 0), int(p.get('kappa') or 0)
            pr.max_err = -1.0 if max_err is None else float(max_err)
            pr.noisy = int(bool(p.get('noisy', False)))
            pr.abs_cutoff = float(p.get('cutoff', 2.718281828459045e-8))
            pr.nops = len(ops)
            pr.op_kind = kind.ctypes.data_as(C.POINTER(C.c_int))
            pr.op_site = site.ctypes.data_as(C.POINTER(C.c_int))
            pr.op_k = kk.ctypes.data_as(C.POINTER(C.c_int))
            pr.op_offset = off.ctypes.data_as(C.POINTER(C.c_int64))
            pr.kraus = _dptr(flat)
            pr.z = _dptr(o['z']) if o['z'] is not None else None
            pr.zz = _dptr(o['zz']) if o['zz'] is not None else None
            pr.discarded = _dptr(o['discarded']) if o['discarded'] is not None else None
            alive += [kind, site, kk, off, flat, vec]
            outs.append((o, n, ntr, pr.dtype))
        nc = len(programs)
        chains = (C.c_void_p * max(1, nc))()
        workers = (C.c_int * max(1, nc))()
        status = (C.c_int * max(1, nc))()
        st = self._lib.mpdo_batch_run(self.handle, nc, arr, chains if keep_chains else None, workers, status)
        results = []
        for i, (o, n, ntr, dt) in enumerate(outs):
            r = {'status': int(status[i]), 'worker': int(workers[i])}
            if o['z'] is not None:
                r['z'] = o['z'][:n]
            if o['zz'] is not None:
                r['zz'] = o['zz'][:n - 1]
            if o['discarded'] is not None:
                r['discarded'] = o['discarded'][:ntr * (n - 1)].reshape(ntr, n - 1)
            if keep_chains and chains[i]:
                r['chain'] = Chain(None, 'complex128' if dt == _lib.MPDO_C128 else 'complex64',
                                   engine=self.engines[int(workers[i])], _handle=C.c_void_p(chains[i]))
            results.append(r)
        check(st)
        return results
