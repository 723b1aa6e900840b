"""Per-block dense / sparse choice models.

The reference decides with a pickled scikit-learn RandomForest over
[rows, cols, density%] (models/density_threshold_spmv.pkl, loaded at
utils/convert_real_to_vbr.py:20 and queried once per block at :58; trained by
studies/find_threshold.py:22-62 on CPU timings from studies/threshold.py).

Models here (all expose choose_dense(features) -> bool[n_blocks], with the
feature rows of convert.block_features: rows, cols, nnz, density, row-nnz
variance, N):

  ThresholdModel   dense iff density% > threshold (the `density` argument of
                   convert_vbr_to_compressed, :51-54).
  RFTableModel     the reference RandomForest, evaluated from a flat tree
                   table (no scikit-learn needed at run time).  The table is
                   extracted once from the reference pickle by
                   models/convert_rf_pkl.py with a whitelisting unpickler.
  MLPModel         the learned cost model: MLP 6 -> 64 -> 64 -> 2 predicting
                   the log2 device time (SM cycles) of the dense and of the
                   sparse form of a block.  A form's cost is its predicted
                   cycles plus, for SpMV (N = 1), kappa_spmv cycles per byte
                   it stores: in a bandwidth-bound launch every byte a block
                   adds also delays the other items sharing DRAM, which its
                   own item cycles do not show.  kappa_spmv is measured with
                   the timings (cycles per byte of large dense blocks).  Dense
                   iff cost_dense < cost_sparse.  Its inference is libsable's
                   batched kernel (sable_mlp_infer), on the GPU only.
default_model() returns the MLP when its weights file exists and a GPU is
present, else the RandomForest table (the reference threshold), as the
fallback.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import pickle

import numpy as np

from . import _lib

MODELS_DIR = pathlib.Path(__file__).resolve().parent / "models"
RF_TABLE = MODELS_DIR / "density_threshold_spmv_rf.npz"
MLP_FILE = MODELS_DIR / "block_cost_mlp.npz"


class ThresholdModel:
    def __init__(self, density: float):
        self.density = float(density)

    def choose_dense(self, feats: np.ndarray) -> np.ndarray:
        pct = feats[:, 2].astype(np.float64) / (feats[:, 0].astype(np.float64) * feats[:, 1]) * 100
        return pct > self.density


class RFTableModel:
    """RandomForestClassifier.predict over [h, w, density%] from flat tables.

    sklearn evaluates trees on float32 inputs with `x[feature] <= threshold`
    and predicts the argmax of the mean of the per-tree leaf class
    fractions; the same rules are applied here."""

    def __init__(self, path: str | os.PathLike = RF_TABLE):
        with np.load(path) as z:
            self.left = z["left"]
            self.right = z["right"]
            self.feature = z["feature"]
            self.threshold = z["threshold"]
            self.value = z["value"]          # [n_nodes, n_classes], leaf class fractions
            self.roots = z["roots"]          # node index of each tree's root
            self.classes = z["classes"]

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.asarray(X, dtype=np.float32).astype(np.float64)
        n = X.shape[0]
        proba = np.zeros((n, self.value.shape[1]))
        rows = np.arange(n)
        for root in self.roots:
            node = np.full(n, root, dtype=np.int64)
            while True:
                active = self.left[node] >= 0
                if not active.any():
                    break
                f = self.feature[node[active]]
                go_left = X[rows[active], f] <= self.threshold[node[active]]
                nxt = np.where(go_left, self.left[node[active]], self.right[node[active]])
                node[active] = nxt
            proba += self.value[node]
        return self.classes[np.argmax(proba, axis=1)]

    def choose_dense(self, feats: np.ndarray) -> np.ndarray:
        pct = (feats[:, 2].astype(np.float64) / (feats[:, 0].astype(np.float64) * feats[:, 1])) * 100
        X = np.stack([feats[:, 0].astype(np.float64), feats[:, 1].astype(np.float64), pct], axis=1)
        return self.predict(X) == 1


_ALLOWED_PREFIXES = ("sklearn.", "numpy")
_ALLOWED_EXACT = {("joblib.numpy_pickle", "NumpyArrayWrapper"), ("_codecs", "encode"),
                  ("joblib.numpy_pickle", "NDArrayWrapper")}


def load_reference_pkl(path: str):
    """Load the reference's joblib pickle, resolving only scikit-learn,
    numpy and joblib array-wrapper globals (anything else raises)."""
    import joblib.numpy_pickle as jnp

    class Restricted(jnp.NumpyUnpickler):
        def find_class(self, module, name):
            if module.startswith(_ALLOWED_PREFIXES) or (module, name) in _ALLOWED_EXACT:
                return super().find_class(module, name)
            raise pickle.UnpicklingError(f"global {module}.{name} is not allowed")

    with open(path, "rb") as fh:
        return Restricted(path, fh, ensure_native_byte_order=True).load()


def rf_to_table(model) -> dict:
    """Flatten a fitted RandomForestClassifier into the arrays RFTableModel reads."""
    lefts, rights, feats, thrs, vals, roots = [], [], [], [], [], []
    base = 0
    for est in model.estimators_:
        t = est.tree_
        roots.append(base)
        left = t.children_left.astype(np.int64)
        right = t.children_right.astype(np.int64)
        lefts.append(np.where(left >= 0, left + base, -1))
        rights.append(np.where(right >= 0, right + base, -1))
        feats.append(np.maximum(t.feature, 0).astype(np.int64))
        thrs.append(t.threshold.astype(np.float64))
        v = t.value[:, 0, :].astype(np.float64)
        vals.append(v / np.maximum(v.sum(axis=1, keepdims=True), 1e-300))
        base += t.node_count
    return {"left": np.concatenate(lefts).astype(np.int32), "right": np.concatenate(rights).astype(np.int32),
            "feature": np.concatenate(feats).astype(np.int8), "threshold": np.concatenate(thrs),
            "value": np.concatenate(vals).astype(np.float32), "roots": np.asarray(roots, dtype=np.int64),
            "classes": np.asarray(model.classes_)}


class MLPModel:
    """Learned block cost model run by libsable's kernels (GPU only)."""

    def __init__(self, params: np.ndarray, mean: np.ndarray, std: np.ndarray, meta: dict | None = None):
        self.params = np.ascontiguousarray(params, dtype=np.float32)
        assert self.params.size == _lib.MLP_NPARAMS
        self.mean = np.ascontiguousarray(mean, dtype=np.float32)
        self.std = np.ascontiguousarray(std, dtype=np.float32)
        self.meta = meta or {}
        self._h = None

    @classmethod
    def load(cls, path: str | os.PathLike = MLP_FILE) -> "MLPModel":
        with np.load(path, allow_pickle=False) as z:
            meta = {k: z[k].item() if z[k].ndim == 0 else z[k] for k in z.files if k not in ("params", "mean", "std")}
            return cls(z["params"], z["mean"], z["std"], meta)

    def save(self, path: str | os.PathLike = MLP_FILE) -> None:
        np.savez(path, params=self.params, mean=self.mean, std=self.std,
                 **{k: np.asarray(v) for k, v in self.meta.items()})

    def handle(self) -> int:
        if self._h is None:
            lib = _lib.load()
            h = ctypes.c_void_p()
            _lib.check(lib.sable_mlp_create(ctypes.byref(h)), "sable_mlp_create")
            _lib.check(lib.sable_mlp_set_params(h, self.params.ctypes.data), "sable_mlp_set_params")
            _lib.check(lib.sable_mlp_set_norm(h, self.mean.ctypes.data, self.std.ctypes.data), "sable_mlp_set_norm")
            self._h = h
        return self._h.value

    def predict(self, feats: np.ndarray) -> np.ndarray:
        """[n, 2] predicted log2 cycles (dense, sparse), computed on the GPU."""
        import torch
        f = torch.as_tensor(np.ascontiguousarray(feats, dtype=np.float32)).cuda()
        out = torch.empty(f.shape[0], 2, dtype=torch.float32, device=f.device)
        if f.shape[0]:
            _lib.check(_lib.load().sable_mlp_infer(self.handle(), f.data_ptr(), f.shape[0], out.data_ptr(),
                                                   torch.cuda.current_stream().cuda_stream), "sable_mlp_infer")
        return out.cpu().numpy()

    @property
    def kappa_spmv(self) -> float:
        return float(self.meta.get("kappa_spmv", 0.0))

    def costs(self, feats: np.ndarray) -> np.ndarray:
        """[n, 2] cost (cycles) of the dense and of the sparse form."""
        return decision_costs(self.predict(feats), feats, self.kappa_spmv)

    def choose_dense(self, feats: np.ndarray) -> np.ndarray:
        c = self.costs(feats)
        return c[:, 0] < c[:, 1]

    def __del__(self):
        try:
            if self._h is not None:
                _lib.load().sable_mlp_destroy(self._h.value)
        except Exception:
            pass


def transform_features(feats: np.ndarray) -> np.ndarray:
    """The kernels' feature transform before normalisation: log2(1 + f) for
    every feature but density (column 3), which is kept as is."""
    f = np.asarray(feats, dtype=np.float64)
    g = np.log2(1.0 + f)
    g[:, 3] = f[:, 3]
    return g


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights (bound sqrt(6 / fan_in)), zero biases, flat order
    W1 b1 W2 b2 W3 b3."""
    rng = np.random.default_rng(seed)
    parts = []
    for out_f, in_f in ((64, 6), (64, 64), (2, 64)):
        lim = np.sqrt(6.0 / in_f)
        parts += [rng.uniform(-lim, lim, size=out_f * in_f), np.zeros(out_f)]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == _lib.MLP_NPARAMS
    return p


def stored_bytes(feats: np.ndarray) -> np.ndarray:
    """[n, 2] bytes the dense and the sparse form of a block store: 4 h w
    dense; CSR 6 nnz in the per-warp SpMV executor's compact records (N = 1),
    8 nnz + 4 (h + 1) in the standard records of SpMM."""
    f = np.asarray(feats, dtype=np.float64)
    sparse = np.where(f[:, 5] == 1, 6 * f[:, 2], 8 * f[:, 2] + 4 * (f[:, 0] + 1))
    return np.stack([4 * f[:, 0] * f[:, 1], sparse], 1)


def decision_costs(log2_cycles: np.ndarray, feats: np.ndarray, kappa_spmv: float) -> np.ndarray:
    """[n, 2] decision cost of both forms from predicted (or measured)
    log2(1 + cycles): cycles, plus kappa_spmv cycles per stored byte for SpMV
    blocks (feature N = 1)."""
    cyc = np.exp2(np.asarray(log2_cycles, dtype=np.float64)) - 1.0
    f = np.asarray(feats, dtype=np.float64)
    bw = np.where((f[:, 5] == 1)[:, None], kappa_spmv * stored_bytes(f), 0.0)
    return cyc + bw


def byte_rule(feats: np.ndarray) -> np.ndarray:
    """Dense iff the dense panel moves no more bytes than the CSR form:
    4 h w <= 8 nnz + 4 (h + 1)."""
    f = np.asarray(feats, dtype=np.float64)
    return 4 * f[:, 0] * f[:, 1] <= 8 * f[:, 2] + 4 * (f[:, 0] + 1)


def regret(dense_choice: np.ndarray, t_dense: np.ndarray, t_sparse: np.ndarray) -> float:
    """sum of the chosen forms' times over the sum of the per-block best, - 1."""
    chosen = np.where(np.asarray(dense_choice, bool), t_dense, t_sparse)
    best = np.minimum(t_dense, t_sparse)
    return float(chosen.sum() / best.sum() - 1.0)


class MLPTrainer:
    """Adam training of the block cost model on the device through
    sable_mlp_train_step (forward, backward and update in libsable's kernels).
    Device memory and the sample shuffle are PyTorch tensors."""

    def __init__(self, params: np.ndarray, mean: np.ndarray, std: np.ndarray, device: int = 0):
        import torch
        self.lib = _lib.load()
        self.dev = torch.device("cuda", device)
        torch.cuda.set_device(self.dev)
        h = ctypes.c_void_p()
        _lib.check(self.lib.sable_mlp_create(ctypes.byref(h)), "sable_mlp_create")
        self._h = h
        self.mean = np.ascontiguousarray(mean, dtype=np.float32)
        self.std = np.ascontiguousarray(std, dtype=np.float32)
        self.set_params(params)
        _lib.check(self.lib.sable_mlp_set_norm(h, self.mean.ctypes.data, self.std.ctypes.data), "sable_mlp_set_norm")

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == _lib.MLP_NPARAMS
        _lib.check(self.lib.sable_mlp_set_params(self._h, p.ctypes.data), "sable_mlp_set_params")

    def params(self) -> np.ndarray:
        out = np.empty(_lib.MLP_NPARAMS, dtype=np.float32)
        _lib.check(self.lib.sable_mlp_get_params(self._h, out.ctypes.data), "sable_mlp_get_params")
        return out

    def _stream(self):
        import torch
        return torch.cuda.current_stream(self.dev).cuda_stream

    def loss_grad(self, feat, target):
        """(loss, grad) of a device batch; both device tensors."""
        import torch
        grad = torch.empty(_lib.MLP_NPARAMS, dtype=torch.float32, device=self.dev)
        loss = torch.empty(1, dtype=torch.float32, device=self.dev)
        _lib.check(self.lib.sable_mlp_loss_grad(self._h, feat.data_ptr(), target.data_ptr(), int(feat.shape[0]),
                                                grad.data_ptr(), loss.data_ptr(), self._stream()),
                   "sable_mlp_loss_grad")
        return loss, grad

    def step(self, feat, target, idx, lr: float, loss=None) -> None:
        _lib.check(self.lib.sable_mlp_train_step(self._h, feat.data_ptr(), target.data_ptr(),
                                                 None if idx is None else idx.data_ptr(),
                                                 int(feat.shape[0] if idx is None else idx.shape[0]), float(lr),
                                                 None if loss is None else loss.data_ptr(), self._stream()),
                   "sable_mlp_train_step")

    def fit(self, feats: np.ndarray, targets: np.ndarray, epochs: int = 40, batch: int = 2048, lr: float = 3e-3,
            lr_final: float = 3e-4, seed: int = 0, log=None, center_output: bool = True) -> list[float]:
        """Mini-batch Adam over (feats, targets) with a per-epoch shuffle and a
        geometric learning-rate decay from lr to lr_final; returns the mean
        batch loss of each epoch.  center_output starts the output biases at
        the mean target (Adam moves a parameter by about lr per step, too
        slowly to travel to log2 cycles from 0)."""
        import torch
        if center_output:
            p = self.params()
            p[-2:] = np.asarray(targets, np.float64).mean(0)
            self.set_params(p)
        f = torch.as_tensor(np.ascontiguousarray(feats, dtype=np.float32), device=self.dev)
        t = torch.as_tensor(np.ascontiguousarray(targets, dtype=np.float32), device=self.dev)
        n = f.shape[0]
        g = torch.Generator(device="cpu").manual_seed(seed)
        losses = torch.zeros(max(1, (n + batch - 1) // batch), dtype=torch.float32, device=self.dev)
        hist = []
        for ep in range(epochs):
            rate = lr * (lr_final / lr) ** (ep / max(1, epochs - 1))
            perm = torch.randperm(n, generator=g).to(torch.int32).to(self.dev)
            nb = 0
            for b0 in range(0, n, batch):
                self.step(f, t, perm[b0:b0 + batch], rate, losses[nb:nb + 1])
                nb += 1
            hist.append(float(losses[:nb].mean()))
            if log:
                log(f"epoch {ep} lr {rate:.2e} loss {hist[-1]:.5f}")
        return hist

    def __del__(self):
        try:
            if self._h:
                self.lib.sable_mlp_destroy(self._h)
        except Exception:
            pass


def default_model():
    """The learned model when its weights and a GPU are present, else the
    reference RandomForest table."""
    if MLP_FILE.exists():
        try:
            import torch
            if torch.cuda.is_available():
                return MLPModel.load(MLP_FILE)
        except ImportError:
            pass
    return RFTableModel(RF_TABLE)
