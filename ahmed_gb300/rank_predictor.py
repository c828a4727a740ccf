"""Learned ACA-rank predictor (8 -> 64 -> 64 -> 1 MLP) trained on the GPU.

The network's forward, backward and Adam kernels are libahx's own
(ahx_mlp_*).  Features are the 8 geometric leaf features of
``HMatrix.features``; the target is log(1 + ACA rank).  Predicted ranks feed
``HMatrix.assemble_hinted``: they size each leaf's ACA workspace and order the
work, while ACA with its own stopping rule still decides every rank.
"""
import ctypes as C

import numpy as np

from ._capi import check, lib, ptr

NFEAT = 8


class RankPredictor:
    def __init__(self, device=0, seed=0):
        h = C.c_void_p()
        check(lib().ahx_mlp_create(device, seed, C.byref(h)))
        self._h = h
        self.nparams = lib().ahx_mlp_nparams()

    def close(self):
        if getattr(self, "_h", None):
            lib().ahx_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        out = np.zeros(self.nparams, np.float32)
        check(lib().ahx_mlp_get_params(self._h, ptr(out)))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().ahx_mlp_set_params(self._h, ptr(p)))

    def set_norm(self, mean, std):
        mean = np.ascontiguousarray(mean, dtype=np.float32)
        std = np.ascontiguousarray(std, dtype=np.float32)
        check(lib().ahx_mlp_set_norm(self._h, ptr(mean), ptr(std)))
        self.mean, self.std = mean, std

    def gradients(self, X, y):
        """Gradient of the mean squared error (targets y, already log-scaled)."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        check(lib().ahx_mlp_gradients(self._h, ptr(X), ptr(y), len(y), ptr(g), C.byref(loss)))
        return g, loss.value

    def fit(self, X, ranks, epochs=30, batch=1024, lr=2e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.log1p(np.asarray(ranks, dtype=np.float32))
        self.set_norm(X.mean(axis=0), X.std(axis=0))
        losses = np.zeros(epochs, np.float32)
        check(lib().ahx_mlp_train(self._h, ptr(X), ptr(np.ascontiguousarray(y)), len(y), epochs,
                                  batch, lr, seed, ptr(losses)))
        return losses

    def predict_log(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(len(X), np.float32)
        if len(X):
            check(lib().ahx_mlp_predict(self._h, ptr(X), len(X), ptr(out)))
        return out

    def predict(self, X):
        # out-of-distribution blocks (e.g. on the diagonal) may predict huge logs
        return np.maximum(np.expm1(np.minimum(self.predict_log(X), 30.0)), 0.0)


def training_set(mats, eps):
    """(features, ACA ranks) of the admissible leaves approximated by ACA in `mats`."""
    Xs, ys = [], []
    for H in mats:
        F = H.features(eps)
        lv = H.leaves()
        r = H.aca_ranks()
        sel = (lv[:, 4] == 1) & (r >= 0)
        Xs.append(F[sel])
        ys.append(r[sel])
    return np.concatenate(Xs), np.concatenate(ys)
