"""ORACLE test infrastructure: warp.types of the numpy Warp stand-in (vector and matrix
types, scalar aliases).  See warp/__init__.py."""
from __future__ import annotations

import numpy as np

float16 = np.float16
float32 = np.float32
float64 = np.float64
int8 = np.int8
int16 = np.int16
int32 = np.int32
int64 = np.int64
uint8 = np.uint8
uint16 = np.uint16
uint32 = np.uint32
uint64 = np.uint64
Float = float32
Int = int32
Scalar = float32


class WArr(np.ndarray):
    """A Warp vector or matrix value: a numpy array with Warp's ``.length``."""

    @property
    def length(self):
        return self.shape[0]


class _CompoundType(type):
    def __call__(cls, *args):
        if not args:
            return np.zeros(cls._inner_shape, dtype=_np_dtype(cls._scalar)).view(WArr)
        if len(args) == 1 and np.ndim(args[0]) > 0:
            return np.array(args[0], dtype=_np_dtype(cls._scalar)).reshape(cls._inner_shape).view(WArr)
        return np.array(args, dtype=_np_dtype(cls._scalar)).reshape(cls._inner_shape).view(WArr)


class VecType(metaclass=_CompoundType):
    _inner_shape = ()
    _scalar = float32


class MatType(metaclass=_CompoundType):
    _inner_shape = ()
    _scalar = float32


_cache: dict = {}


def vector(length, dtype=float32):
    """warp.types.vector(length, dtype): the vector type."""
    if dtype is float:
        dtype = float32
    elif dtype is int:
        dtype = int32
    key = ("vec", int(length), np.dtype(dtype).str)
    if key not in _cache:
        _cache[key] = _CompoundType(f"vec{int(length)}_{np.dtype(dtype).name}", (VecType,),
                                    {"_inner_shape": (int(length),), "_scalar": dtype, "_length_": int(length),
                                     "dtype": dtype})
    return _cache[key]


def matrix(shape, dtype=float32):
    """warp.types.matrix / warp.mat(shape, dtype): the matrix type."""
    if dtype is float:
        dtype = float32
    elif dtype is int:
        dtype = int32
    shape = tuple(int(s) for s in shape)
    key = ("mat", shape, np.dtype(dtype).str)
    if key not in _cache:
        _cache[key] = _CompoundType(f"mat{shape[0]}{shape[1]}_{np.dtype(dtype).name}", (MatType,),
                                    {"_inner_shape": shape, "_scalar": dtype, "_shape_": shape, "dtype": dtype})
    return _cache[key]


mat = matrix
vec2 = vector(2, float32)
vec3 = vector(3, float32)
vec4 = vector(4, float32)
vec2f, vec3f, vec4f = vec2, vec3, vec4
vec3d = vector(3, float64)


def _is_struct(t) -> bool:
    return bool(getattr(t, "_warp_struct", False))


def _np_dtype(t):
    """The numpy dtype of a Warp element type (vector/matrix: its scalar)."""
    if t is None:
        return np.dtype(np.float32)
    if t is float:
        return np.dtype(np.float32)
    if t is int:
        return np.dtype(np.int32)
    if isinstance(t, type) and issubclass(t, (VecType, MatType)):
        return np.dtype(t._scalar)
    return np.dtype(t)


def _zero_of(t):
    if isinstance(t, type) and issubclass(t, (VecType, MatType)):
        return t()
    if _is_struct(t):
        return t()
    if t is None:
        return None
    try:
        return _np_dtype(t).type(0)
    except TypeError:
        return None
