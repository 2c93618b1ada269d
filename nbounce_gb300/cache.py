"""Radiance cache: binding of the ``nb_cache_*`` C ABI.

The network is a 64 -> 5 x 64 (ReLU) -> 3 MLP (bias-free; encoded input 62 is a constant 1)
evaluated and trained by the library's BF16 tensor-core kernels.  ``weights`` is the flat FP32
array the kernels update: layer ``l < 5`` is ``W_l[out][in]`` (64 x 64) at ``l * 4096``, the
output layer ``W_5`` (16 x 64, rows 3..15 zero) at 20480, so ``relu(x @ W_l.T)`` is one layer.

Device arrays are passed as objects with ``data_ptr()`` (torch CUDA tensors) or raw integer
addresses.  ``Pathtracer.set_cache`` attaches a cache: every render call is then one frame
whose paths end in cache lookups and whose training paths train the cache.
"""
import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check, lib, ptr

N_PARAMS = L.NB_CACHE_PARAMS
N_INPUTS = L.NB_CACHE_INPUTS
LAYER_SHAPES = [(64, 64)] * 5 + [(16, 64)]


def _dptr(x):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    return C.c_void_p(int(x))


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


def split_layers(w):
    """Flat weights -> list of per-layer [out][in] arrays (views)."""
    out, off = [], 0
    for o, i in LAYER_SHAPES:
        out.append(w[off:off + o * i].reshape(o, i))
        off += o * i
    return out


def default_config():
    c = L.NbCacheConfig()
    lib().nb_cache_default_config(C.byref(c))
    return c


class RadianceCache:
    """nb_cache handle.  Keyword arguments override fields of the default configuration
    (learning_rate, beta1, beta2, epsilon, spread, train_records, train_steps,
    extra_vertices, seed)."""

    def __init__(self, **overrides):
        cfg = default_config()
        for k, v in overrides.items():
            if not hasattr(cfg, k):
                raise TypeError(f"unknown cache setting {k!r}")
            setattr(cfg, k, v)
        h = C.c_void_p()
        check(lib().nb_cache_create(C.byref(cfg), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    @property
    def config(self):
        c = L.NbCacheConfig()
        check(lib().nb_cache_get_config(self._h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in L.NbCacheConfig._fields_}

    def set_bounds(self, lo, hi):
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        check(lib().nb_cache_set_bounds(self._h, ptr(lo), ptr(hi)))

    def get_weights(self):
        w = np.zeros(N_PARAMS, np.float32)
        check(lib().nb_cache_get_weights(self._h, ptr(w), N_PARAMS))
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32).ravel()
        check(lib().nb_cache_set_weights(self._h, ptr(w), w.size))

    def encode(self, vertices_dev, n, out_dev, stream=None):
        check(lib().nb_cache_encode(self._h, _dptr(vertices_dev), int(n), _dptr(out_dev), _stream(stream)))

    def infer(self, inputs_dev, n, out_dev, stream=None):
        check(lib().nb_cache_infer(self._h, _dptr(inputs_dev), int(n), _dptr(out_dev), _stream(stream)))

    def gradient(self, inputs_dev, targets_dev, n, grad_dev, stream=None):
        loss = C.c_float()
        check(lib().nb_cache_gradient(self._h, _dptr(inputs_dev), _dptr(targets_dev), int(n), _dptr(grad_dev),
                                      C.byref(loss), _stream(stream)))
        return float(loss.value)

    def train_step(self, inputs_dev, targets_dev, n, stream=None):
        loss = C.c_float()
        check(lib().nb_cache_train_step(self._h, _dptr(inputs_dev), _dptr(targets_dev), int(n), C.byref(loss),
                                        _stream(stream)))
        return float(loss.value)

    def stats(self, stream=None):
        s = L.NbCacheStats()
        check(lib().nb_cache_get_stats(self._h, C.byref(s), _stream(stream)))
        return {k: getattr(s, k) for k, _ in L.NbCacheStats._fields_}

    def close(self):
        if self._h:
            lib().nb_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
