"""Python handle of the C-ABI multilayer perceptron (pbag_mlp_*): FP32
training kernels, FP32 and BF16 tensor-core inference of the library, data as
device addresses."""
import ctypes as C

import numpy as np

from . import _lib


def _l():
    lib = _lib.load()
    if not getattr(lib, "_mlp_bound", False):
        P = C.POINTER
        lib.pbag_mlp_create.argtypes = [C.c_int, P(C.c_int), C.c_int, P(C.c_void_p)]
        lib.pbag_mlp_destroy.argtypes = [C.c_void_p]
        lib.pbag_mlp_param_count.argtypes = [C.c_void_p]
        lib.pbag_mlp_param_count.restype = C.c_int64
        lib.pbag_mlp_set_params.argtypes = [C.c_void_p, P(C.c_float)]
        lib.pbag_mlp_get_params.argtypes = [C.c_void_p, P(C.c_float), P(C.c_float)]
        lib.pbag_mlp_forward.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        lib.pbag_mlp_infer.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        lib.pbag_mlp_train_step.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                            C.c_int, P(C.c_float)]
        lib._mlp_bound = True
    return lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class MLP:
    """dims = [d_0, ..., d_L]; SiLU hidden layers, linear output."""

    def __init__(self, dims, device=0):
        lib = _l()
        self.dims = list(dims)
        arr = (C.c_int * len(self.dims))(*self.dims)
        h = C.c_void_p()
        _lib._check(lib.pbag_mlp_create(int(device), arr, len(self.dims) - 1, C.byref(h)), "pbag_mlp_create")
        self._h = h
        self.nparams = int(lib.pbag_mlp_param_count(h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _l().pbag_mlp_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def init_params(self, seed=0):
        """He-style initialisation (the same layout the library uses)."""
        rng = np.random.default_rng(seed)
        p = []
        for din, dout in zip(self.dims[:-1], self.dims[1:]):
            p.append(rng.normal(0.0, np.sqrt(2.0 / din), size=(dout, din)).ravel())
            p.append(np.zeros(dout))
        params = np.concatenate(p).astype(np.float32)
        self.set_params(params)
        return params

    def set_params(self, params):
        params = np.ascontiguousarray(params, dtype=np.float32)
        assert params.size == self.nparams
        _lib._check(_l().pbag_mlp_set_params(self._h, _fp(params)), "pbag_mlp_set_params")

    def params(self, grads=False):
        p = np.zeros(self.nparams, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32) if grads else None
        _lib._check(_l().pbag_mlp_get_params(self._h, _fp(p), _fp(g) if grads else None), "pbag_mlp_get_params")
        return (p, g) if grads else p

    def forward(self, n, d_x, d_y):
        _lib._check(_l().pbag_mlp_forward(self._h, int(n), C.c_void_p(d_x), C.c_void_p(d_y)), "pbag_mlp_forward")

    def infer(self, n, d_x, d_y):
        """BF16 inference on the tensor cores (pbag_mlp_infer)."""
        _lib._check(_l().pbag_mlp_infer(self._h, int(n), C.c_void_p(d_x), C.c_void_p(d_y)), "pbag_mlp_infer")

    def train_step(self, n, d_x, d_t, d_mask=0, lr=1e-3, update=True):
        loss = C.c_float()
        _lib._check(_l().pbag_mlp_train_step(self._h, int(n), C.c_void_p(d_x), C.c_void_p(d_t),
                                             C.c_void_p(d_mask or None), float(lr), int(bool(update)),
                                             C.byref(loss)), "pbag_mlp_train_step")
        return float(loss.value)
