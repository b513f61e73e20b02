"""ORACLE test infrastructure: a numpy stand-in for the subset of NVIDIA Warp (warp-lang)
that warp_cfd's solver path uses, so the unmodified warp_cfd sources run on a CPU without
warp-lang.  Not part of the product; only tests/golden/make_reference_golden.py puts it on
sys.path.

Semantics kept from Warp:
* ``@wp.kernel`` functions run once per thread index of ``wp.launch(dim=...)``, in
  row-major launch order (Warp's CPU backend runs a launch's threads sequentially), with
  ``wp.tid()`` returning the current index (an int for 1-D launches, a tuple otherwise);
* scalar arithmetic in the array's own precision (numpy scalars of float32 / float64);
* arrays of vectors / matrices index to vectors / matrices that write through to the
  array; arrays of structs hold mutable struct objects;
* ``wp.atomic_add`` adds in place (sequential threads make it an ordinary add).
"""
from __future__ import annotations

import itertools
import types as _pytypes

import numpy as np

from . import types  # noqa: F401  (warp.types)
from .types import (WArr, VecType, MatType, vector, matrix, mat, _is_struct, _np_dtype, _zero_of,  # noqa: F401
                    float16, float32, float64, int8, int16, int32, int64, uint8, uint16, uint32, uint64,
                    vec2, vec3, vec4, vec2f, vec3f, vec4f, vec3d, Float, Int, Scalar)

__version__ = "stand-in"

config = _pytypes.SimpleNamespace(mode="release", verify_fp=False, verbose=False, print_launches=False)

_tid = 0


def init():
    return None


def clear_kernel_cache():
    return None


def set_device(*a, **k):
    return None


def synchronize():
    return None


def get_device(*a, **k):
    return "cpu"


# --------------------------------------------------------------------------- arrays
class array:
    """A Warp array over a numpy buffer.  ``dtype`` is the element type (a numpy scalar
    class, a VecType/MatType or a struct class); ``shape`` the outer shape."""

    def __class_getitem__(cls, item):
        return cls

    def __init__(self, data=None, dtype=None, shape=None, device=None, ndim=None, copy=True, requires_grad=False,
                 owner=False, **kw):
        if dtype is float:
            dtype = float32
        elif dtype is int:
            dtype = int32
        elif dtype is bool:
            dtype = np.bool_
        self._annotation = data is None and shape is None
        if data is None and shape is None:
            # a type annotation such as wp.array(dtype=float) or wp.array(ndim=4, dtype=...)
            self.dtype = dtype
            self.ndim = ndim or 1
            self.shape = (0,) * self.ndim
            self._data = None
            return
        if data is not None:
            if isinstance(data, array):
                data = data._data
            if dtype is None:
                arr = np.asarray(data)
                dtype = arr.dtype.type
            self.dtype = dtype
            if _is_struct(dtype):
                src = np.asarray(data, dtype=object)
                self._data = src.copy() if copy else src
                self.shape = self._data.shape
            else:
                inner = getattr(dtype, "_inner_shape", ())
                arr = np.array(data, dtype=_np_dtype(dtype), copy=True if copy else None)
                if inner:
                    outer = arr.shape[:arr.ndim - len(inner)]
                    if arr.shape[len(outer):] != tuple(inner):
                        arr = arr.reshape(tuple(outer) + tuple(inner))
                    self.shape = tuple(outer)
                else:
                    self.shape = arr.shape
                self._data = arr
        else:
            if isinstance(shape, (int, np.integer)):
                shape = (int(shape),)
            shape = tuple(int(s) for s in shape)
            if dtype is None:
                dtype = float32
            self.dtype = dtype
            self.shape = shape
            if _is_struct(dtype):
                self._data = np.empty(shape, dtype=object)
                for idx in np.ndindex(*shape):
                    self._data[idx] = dtype()
            else:
                inner = tuple(getattr(dtype, "_inner_shape", ()))
                self._data = np.zeros(shape + inner, dtype=_np_dtype(dtype))
        self.ndim = len(self.shape)

    # ---- element access (kernels and host)
    def _full(self, key):
        return key if isinstance(key, tuple) else (key,)

    def __getitem__(self, key):
        k = self._full(key)
        if _is_struct(self.dtype):
            return self._data[k]
        v = self._data[k]
        if isinstance(v, np.ndarray):
            if len(k) == self.ndim and getattr(self.dtype, "_inner_shape", ()):
                return v.view(WArr)
            # a sub-array (partial index)
            sub = array.__new__(array)
            sub.dtype = self.dtype
            sub._data = v
            sub._annotation = False
            sub.shape = v.shape[:v.ndim - len(getattr(self.dtype, "_inner_shape", ()))]
            sub.ndim = len(sub.shape)
            return sub
        return v

    def __setitem__(self, key, value):
        k = self._full(key)
        if _is_struct(self.dtype):
            self._data[k] = value
            return
        if isinstance(value, array):
            value = value._data
        self._data[k] = value

    # ---- host API
    @property
    def size(self):
        return int(np.prod(self.shape)) if self.shape else 1

    def __len__(self):
        return self.shape[0]

    @property
    def device(self):
        return "cpu"

    def numpy(self):
        return self._data

    def list(self):
        return list(self._data)

    def zero_(self):
        if _is_struct(self.dtype):
            for idx in np.ndindex(*self.shape):
                self._data[idx] = self.dtype()
        else:
            self._data[...] = 0

    def fill_(self, value):
        self._data[...] = value

    def assign(self, src):
        self._data[...] = src._data if isinstance(src, array) else src

    def flatten(self):
        out = array.__new__(array)
        out.dtype = self.dtype
        inner = tuple(getattr(self.dtype, "_inner_shape", ()))
        out._data = self._data.reshape((-1,) + inner)
        out._annotation = False
        out.shape = (out._data.shape[0],)
        out.ndim = 1
        return out

    def reshape(self, shape):
        if isinstance(shape, (int, np.integer)):
            shape = (int(shape),)
        out = array.__new__(array)
        out.dtype = self.dtype
        inner = tuple(getattr(self.dtype, "_inner_shape", ()))
        out._data = self._data.reshape(tuple(shape) + inner)
        out._annotation = False
        out.shape = out._data.shape[:out._data.ndim - len(inner)]
        out.ndim = len(out.shape)
        return out

    def _like(self, data):
        out = array.__new__(array)
        out.dtype = self.dtype
        out._data = data
        out._annotation = False
        out.shape = self.shape
        out.ndim = self.ndim
        return out

    def _scalar(self, v):
        return v._data if isinstance(v, array) else v

    def __add__(self, o):
        return self._like((self._data + self._scalar(o)).astype(self._data.dtype, copy=False))

    def __radd__(self, o):
        return self.__add__(o)

    def __sub__(self, o):
        return self._like((self._data - self._scalar(o)).astype(self._data.dtype, copy=False))

    def __rsub__(self, o):
        return self._like((self._scalar(o) - self._data).astype(self._data.dtype, copy=False))

    def __mul__(self, o):
        return self._like((self._data * self._scalar(o)).astype(self._data.dtype, copy=False))

    def __rmul__(self, o):
        return self.__mul__(o)

    def __truediv__(self, o):
        return self._like((self._data / self._scalar(o)).astype(self._data.dtype, copy=False))

    def __neg__(self):
        return self._like(-self._data)

    def __iadd__(self, o):
        self._data += self._scalar(o)
        return self

    def __isub__(self, o):
        self._data -= self._scalar(o)
        return self

    def __imul__(self, o):
        self._data *= self._scalar(o)
        return self

    def __repr__(self):
        return f"warp_stand_in.array(shape={self.shape}, dtype={getattr(self.dtype, '__name__', self.dtype)})"


def array1d(*a, **k):
    k.setdefault("ndim", 1)
    return array(*a, **k)


def array2d(*a, **k):
    k.setdefault("ndim", 2)
    return array(*a, **k)


def array3d(*a, **k):
    k.setdefault("ndim", 3)
    return array(*a, **k)


def array4d(*a, **k):
    k.setdefault("ndim", 4)
    return array(*a, **k)


def zeros(shape=None, dtype=float, device=None, requires_grad=False, **kw):
    if shape is None:
        shape = kw.pop("n")
    return array(shape=shape, dtype=dtype)


def empty(shape=None, dtype=float, device=None, requires_grad=False, **kw):
    return zeros(shape, dtype)


def zeros_like(a, device=None, requires_grad=None):
    return array(shape=a.shape, dtype=a.dtype)


def empty_like(a, device=None, requires_grad=None):
    return zeros_like(a)


def clone(a, device=None):
    return a._like(a._data.copy())


def copy(dest, src, dest_offset=0, src_offset=0, count=0):
    n = count or src.size
    dest._data.reshape(-1)[dest_offset:dest_offset + n] = src._data.reshape(-1)[src_offset:src_offset + n]


def from_numpy(arr, dtype=None, shape=None, device=None):
    return array(data=arr, dtype=dtype)


def dtype_from_numpy(t):
    return np.dtype(t).type


def dtype_to_numpy(t):
    return np.dtype(_np_dtype(t))


# --------------------------------------------------------------------------- structs
def struct(cls):
    """A Warp struct: members from the class annotations, zero-initialised; vector and
    matrix members are mutable numpy views; assignment copies (value semantics)."""
    members = dict(getattr(cls, "__annotations__", {}))

    class _Struct:
        __slots__ = tuple(members)
        _warp_struct = True
        vars = members

        def __init__(self):
            for name, t in members.items():
                object.__setattr__(self, name, _zero_of(t))

        def __setattr__(self, name, value):
            t = members.get(name)
            if t is None:
                raise AttributeError(f"struct {cls.__name__} has no member {name}")
            inner = getattr(t, "_inner_shape", ())
            if inner:
                arr = np.array(value._data if isinstance(value, array) else value, dtype=_np_dtype(t)).reshape(inner)
                object.__setattr__(self, name, arr.view(WArr))
            elif _is_struct(t):
                object.__setattr__(self, name, value)
            else:
                object.__setattr__(self, name, _np_dtype(t).type(value) if t is not None else value)

    _Struct.__name__ = cls.__name__
    _Struct.__qualname__ = cls.__qualname__
    return _Struct


# --------------------------------------------------------------------------- kernels
class Kernel:
    def __init__(self, func):
        self.func = func
        self.key = func.__name__
        self.__name__ = func.__name__

    def __call__(self, *a, **k):
        return self.func(*a, **k)


def kernel(func=None, enable_backward=None, module=None):
    if func is None:
        return lambda f: Kernel(f)
    return Kernel(func)


def func(f=None, **kw):
    if f is None:
        return lambda g: g
    return f


def overload(kernel_or_func, arg_types=None):
    return kernel_or_func


def static(x):
    return x


def tid():
    return _tid


def launch(kernel, dim, inputs=(), outputs=(), adj_inputs=None, adj_outputs=None, device=None, stream=None,
           adjoint=False, record_tape=True, record_cmd=False, max_blocks=0, block_dim=256):
    global _tid
    f = kernel.func if isinstance(kernel, Kernel) else kernel
    args = list(inputs) + list(outputs)
    if isinstance(dim, (int, np.integer)):
        dims = (int(dim),)
    else:
        dims = tuple(int(d) for d in dim)
    if len(dims) == 1:
        for i in range(dims[0]):
            _tid = i
            f(*args)
    else:
        for idx in itertools.product(*[range(d) for d in dims]):
            _tid = idx
            f(*args)
    _tid = 0


# --------------------------------------------------------------------------- builtins
def atomic_add(arr, *args):
    *idx, value = args
    k = tuple(int(i) for i in idx)
    old = arr._data[k].copy() if isinstance(arr._data[k], np.ndarray) else arr._data[k]
    if isinstance(value, np.ndarray):
        arr._data[k] += value
    else:
        arr._data[k] = arr._data[k] + value
    return old


def atomic_sub(arr, *args):
    *idx, value = args
    return atomic_add(arr, *idx, -value)


def length(v):
    return np.sqrt(np.dot(v, v))


def length_sq(v):
    return np.dot(v, v)


def dot(a, b):
    return np.dot(a, b)


def cross(a, b):
    return np.cross(a, b).view(WArr)


def normalize(v):
    return (v / length(v)).view(WArr)


def sub(a, b):
    return a - b


def add(a, b):
    return a + b


def mul(a, b):
    return a * b


def div(a, b):
    return a / b


def neg(a):
    return -a


def mod(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
        q = abs(int(a)) % abs(int(b))
        return type(a)(q if a >= 0 else -q)
    return np.fmod(a, b)


def abs(x):  # noqa: A001 - Warp's builtin name
    return np.abs(x)


def sqrt(x):
    return np.sqrt(x)


def min(a, b):  # noqa: A001
    return np.minimum(a, b)


def max(a, b):  # noqa: A001
    return np.maximum(a, b)


def select(cond, a, b):
    return b if cond else a


def where(cond, a, b):
    return a if cond else b


def printf(fmt, *args):
    return None


def vector(*args, length=None, dtype=None):
    """The in-kernel vector constructor: wp.vector(a, b, c) or wp.vector(length=n, dtype=T)."""
    if args:
        dt = _np_dtype(dtype) if dtype is not None else np.result_type(*[np.asarray(a).dtype for a in args])
        return np.array(args, dtype=dt).view(WArr)
    return np.zeros(int(length), dtype=_np_dtype(dtype if dtype is not None else float32)).view(WArr)
