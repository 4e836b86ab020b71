"""Python binding of the neural radiance cache entry points (nr_nrc_*)."""
import ctypes

import numpy as np

from ._lib import _ptr, check, lib

INPUTS = 80
HIDDEN = 64
OFF = {}
_o = 0
for _name, _size in (("W0", 64 * 80), ("b0", 64), ("W1", 64 * 64), ("b1", 64), ("W2", 64 * 64), ("b2", 64),
                     ("W3", 64 * 64), ("b3", 64), ("W4", 8 * 64), ("b4", 8)):
    OFF[_name] = (_o, _size)
    _o += _size
NUM_PARAMS = _o


def _bind():
    return lib()


class Cache:
    def __init__(self, params=""):
        self.L = _bind()
        h = ctypes.c_void_p()
        check(self.L.nr_nrc_create(params.encode(), ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            check(self.L.nr_nrc_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        p = np.zeros(NUM_PARAMS, np.float32)
        check(self.L.nr_nrc_get_params(self._h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == NUM_PARAMS
        check(self.L.nr_nrc_set_params(self._h, _ptr(p)))

    # nr_nrc_get_state / nr_nrc_set_state selectors
    STATE = dict(params=0, grad=1, m=2, v=3, ema=4, infer=5, params_bf16=6, infer_bf16=7, step=8)

    def get_state(self, which):
        """One array of the training state (include/nuray.h NR_NRC_STATE_*);
        'step' returns the Adam step count."""
        k = self.STATE[which]
        out = np.zeros(1 if which == "step" else NUM_PARAMS, np.float32)
        check(self.L.nr_nrc_get_state(self._h, k, _ptr(out)))
        return int(out[0]) if which == "step" else out

    def set_state(self, which, value):
        k = self.STATE[which]
        a = np.array([value], np.float32) if which == "step" else np.ascontiguousarray(value, np.float32)
        assert which == "step" or a.size == NUM_PARAMS
        check(self.L.nr_nrc_set_state(self._h, k, _ptr(a)))

    def infer(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, INPUTS)
        out = np.zeros((x.shape[0], 3), np.float32)
        check(self.L.nr_nrc_infer(self._h, x.shape[0], _ptr(x), _ptr(out)))
        return out

    def gradient(self, x, y):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, INPUTS)
        y = np.ascontiguousarray(y, np.float32).reshape(-1, 3)
        g = np.zeros(NUM_PARAMS, np.float32)
        loss = ctypes.c_float()
        check(self.L.nr_nrc_gradient(self._h, x.shape[0], _ptr(x), _ptr(y), _ptr(g), ctypes.byref(loss)))
        return g, loss.value

    def train_step(self, x, y):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, INPUTS)
        y = np.ascontiguousarray(y, np.float32).reshape(-1, 3)
        loss = ctypes.c_float()
        check(self.L.nr_nrc_train_step(self._h, x.shape[0], _ptr(x), _ptr(y), ctypes.byref(loss)))
        return loss.value

    def attach(self, scene):
        check(self.L.nr_scene_attach_nrc(scene._h, self._h))


def unpack(p):
    """Parameter vector -> dict of numpy arrays (W4 / b4 keep their 8 padded rows)."""
    out = {}
    for k, (o, n) in OFF.items():
        a = p[o:o + n]
        if k.startswith("W"):
            a = a.reshape(-1, INPUTS if k == "W0" else HIDDEN)
        out[k] = a
    return out
