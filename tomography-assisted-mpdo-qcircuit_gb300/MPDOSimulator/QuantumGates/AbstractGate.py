"""Gate base classes (reference: QuantumGates/AbstractGate.py:13-99).

Gate tensors are built with differentiable torch ops (the reference rebuilds
them through ``torch.tensor(data=...)``, which detaches the angle from the
graph); index order is [out, in] for one qubit and [out0, out1, in0, in1] for
two qubits, as in the reference.
"""
from abc import ABC, abstractmethod
from typing import Optional

import numpy as np
import torch
from torch import Tensor, nn


class Truncate(nn.Module):
    def __init__(self):
        super().__init__()
        self.name = 'truncate'

    def forward(self, *args, **kwargs):
        pass


class Barrier(nn.Module):
    def __init__(self):
        super().__init__()
        self.name = 'barrier'

    def forward(self, *args, **kwargs):
        pass


_MODULE_STATE = None
_MODULE_FLAGS = None


def _module_state() -> dict:
    global _MODULE_STATE
    if _MODULE_STATE is None:
        _MODULE_STATE = dict(nn.Module().__dict__)
    return _MODULE_STATE


def _module_init(obj: nn.Module) -> None:
    """``nn.Module.__init__`` for a gate: its flags now, its (empty)
    parameter / buffer / submodule / hook containers on first access
    (``QuantumGate.__getattr__``).  A circuit builds one gate module per gate;
    a dozen fresh containers per gate made the cyclic garbage collector run
    through the growing circuit over and over, half of the build time.  The
    flags are picked out of nn.Module's state once per process."""
    global _MODULE_FLAGS
    if _MODULE_FLAGS is None:
        _MODULE_FLAGS = {k: v for k, v in _module_state().items() if not isinstance(v, (dict, set, list))}
    obj.__dict__.update(_MODULE_FLAGS)


class QuantumGate(ABC, nn.Module):
    """Base class for quantum gates (AbstractGate.py:31-99)."""

    def __init__(self, ideal: Optional[bool] = True, dtype=torch.complex64, device='cpu'):
        _module_init(self)
        # plain attributes, set without the per-attribute module check
        self.__dict__.update(para=None, _ideal=ideal, dtype=dtype, device=device)

    def __getattr__(self, name):
        # nn.Module's per-instance containers, created on first use (each
        # gate gets its own, as after nn.Module.__init__)
        proto = _module_state().get(name)
        if isinstance(proto, (dict, set, list)):
            value = proto.copy()
            self.__dict__[name] = value
            return value
        return nn.Module.__getattr__(self, name)

    def __setattr__(self, name, value):
        # gates hold no parameters, buffers or submodules: plain attributes
        # bypass nn.Module's registration checks, which otherwise dominate the
        # cost of building circuits of many gates
        if isinstance(value, nn.Module):
            self._modules                    # noqa: B018 -- create the container nn.Module registers into
            nn.Module.__setattr__(self, name, value)
        else:
            object.__setattr__(self, name, value)

    def _check_Para_Tensor(self, *parameters):
        """AbstractGate.py:42-51 casts angles to the circuit's complex dtype, so
        the trigonometry runs at that precision (an angle given as a float32
        tensor is widened first).  Angles stay real here, at the matching real
        precision, which gives the same values and keeps them differentiable.
        An angle given as a number stays in host memory: the engine takes gate
        matrices from the host, so a device copy would only cost a transfer
        each way per gate (``tensor`` still returns the matrix on ``device``)."""
        rdt = torch.float64 if self.dtype == torch.complex128 else torch.float32

        def conv(p):
            tp = type(p)
            if tp is float or tp is int:           # the common case first
                return torch.tensor(float(p), dtype=rdt)
            if isinstance(p, Tensor):
                return p.to(device=self.device, dtype=self.dtype if p.is_complex() else rdt)
            if isinstance(p, (float, int)):
                return torch.tensor(float(p), dtype=rdt)
            raise ValueError(f'Invalid type for gate parameter: {type(p)}')
        ps = [conv(p) for p in parameters]
        return ps if len(parameters) > 1 else ps[0]

    def _mat(self, rows):
        """Stack a nested list of (possibly tensor-valued) entries into a complex
        matrix, keeping autograd through tensor entries."""
        cdt = self.dtype
        out = []
        for row in rows:
            out.append(torch.stack([torch.as_tensor(x, device=self.device).to(cdt) for x in row]))
        return torch.stack(out)

    @property
    @abstractmethod
    def name(self):
        pass

    @property
    @abstractmethod
    def tensor(self):
        pass

    @property
    @abstractmethod
    def rank(self):
        pass

    @property
    @abstractmethod
    def dimension(self):
        pass

    @property
    @abstractmethod
    def single(self) -> bool:
        pass

    @property
    @abstractmethod
    def variational(self) -> bool:
        pass

    @property
    def para(self):
        return self._para

    @para.setter
    def para(self, para):
        self._para = para

    @property
    def ideal(self) -> Optional[bool]:
        return self._ideal

    @ideal.setter
    def ideal(self, value: Optional[bool]):
        if not isinstance(value, bool):
            raise ValueError('Value must be bool.')
        self._ideal = value


def _cexp(x):
    """exp(1j * x) for a real tensor/float, differentiable."""
    x = torch.as_tensor(x, dtype=torch.float64) if not isinstance(x, Tensor) else x
    if x.is_complex():
        return torch.exp(1j * x)
    return torch.complex(torch.cos(x), torch.sin(x))


class _Fixed(QuantumGate):
    """A constant gate defined by a matrix literal."""
    _NAME = ''
    _DATA = None
    _SINGLE = True

    def __init__(self, ideal: Optional[bool] = None, dtype=torch.complex64, device='cpu'):
        super().__init__(ideal=ideal, dtype=dtype, device=device)

    @property
    def name(self):
        return self._NAME

    @property
    def tensor(self):
        t = torch.tensor(self._DATA, dtype=self.dtype, device=self.device)
        return t if self._SINGLE else t.reshape(2, 2, 2, 2)

    _NP_CACHE = {}

    def numpy_tensor(self):
        """The matrix as complex128 numpy, its entries rounded to ``dtype``
        (the values ``tensor`` holds), built once per gate class and dtype."""
        key = (type(self), self.dtype)
        t = _Fixed._NP_CACHE.get(key)
        if t is None:
            np_dt = np.complex64 if self.dtype == torch.complex64 else np.complex128
            t = np.asarray(self._DATA, dtype=np_dt).astype(np.complex128)
            t = t if self._SINGLE else t.reshape(2, 2, 2, 2)
            t.setflags(write=False)
            _Fixed._NP_CACHE[key] = t
        return t

    @property
    def rank(self):
        return 2 if self._SINGLE else 4

    @property
    def dimension(self):
        return [2, 2] if self._SINGLE else [[2, 2], [2, 2]]

    @property
    def single(self) -> bool:
        return self._SINGLE

    @property
    def variational(self) -> bool:
        return False


class _Param(QuantumGate):
    """A parameterised gate; subclasses define ``_build()``."""
    _NAME = ''
    _SINGLE = True

    @property
    def name(self):
        return self._NAME

    @property
    def rank(self):
        return 2 if self._SINGLE else 4

    @property
    def dimension(self):
        return [2, 2] if self._SINGLE else [[2, 2], [2, 2]]

    @property
    def single(self) -> bool:
        return self._SINGLE

    @property
    def variational(self) -> bool:
        return True

    @property
    def tensor(self):
        t = self._build()
        return t if self._SINGLE else t.reshape(2, 2, 2, 2)

    def numpy_tensor(self):
        """The gate as a complex128 numpy array, for the engine (which takes
        host Kraus tensors).  Gates that define ``_build_np`` evaluate it on
        plain floats when no parameter needs a gradient (the angles rounded to
        the circuit's real precision, as ``_check_Para_Tensor`` stores them);
        otherwise the autograd-capable ``tensor`` is converted."""
        params = self.para if isinstance(self.para, (list, tuple)) else [self.para]
        if hasattr(self, '_build_np') and all(isinstance(q, Tensor) and not q.requires_grad and not q.is_complex()
                                              for q in params):
            t = self._build_np(*[float(q) for q in params])
            return t if self._SINGLE else t.reshape(2, 2, 2, 2)
        return self.tensor.detach().to('cpu', torch.complex128).numpy()
