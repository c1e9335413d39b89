"""CPU oracle of the ARF network: forward, softmax cross-entropy and backward in FP64.

Test infrastructure only: the tests compare the GPU network (BF16 tensor-core
GEMMs with FP32 accumulation) with this restatement.  The network restates
the garf ARF model the reference's ARFActor evaluates
(opengate/actors/arfactors.py:299-415; garf itself is not part of the
reference tree): x = standardised (theta deg, phi deg, E MeV), three hidden
layers of 128 ReLU units, n_classes logits, softmax; class 0 = no energy
window.  Parameter layout (FP32 array of 35600): W1[128][3], b1[128],
W2[128][128], b2[128], W3[128][128], b3[128], W4[16][128], b4[16].

``bf16=True`` rounds to bfloat16 where the GPU kernels store BF16 (weights of
layers 2-4, the hidden activations, the output gradient and the hidden
gradients), everything else in FP64; ``bf16=False`` is FP64 throughout.
"""

import numpy as np

HID = 128
OUT_PAD = 16
OFF = {}
_o = 0
for _name, _size in (("W1", HID * 3), ("b1", HID), ("W2", HID * HID), ("b2", HID), ("W3", HID * HID), ("b3", HID),
                     ("W4", OUT_PAD * HID), ("b4", OUT_PAD)):
    OFF[_name] = (_o, _size)
    _o += _size
N_PARAMS = _o
SHAPES = {"W1": (HID, 3), "b1": (HID,), "W2": (HID, HID), "b2": (HID,), "W3": (HID, HID), "b3": (HID,),
          "W4": (OUT_PAD, HID), "b4": (OUT_PAD,)}


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    return {k: p[o:o + n].reshape(SHAPES[k]) for k, (o, n) in OFF.items()}


def pack(d):
    out = np.zeros(N_PARAMS, dtype=np.float64)
    for k, (o, n) in OFF.items():
        out[o:o + n] = np.asarray(d[k], dtype=np.float64).reshape(-1)
    return out


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def features(rows, mean, std):
    """Standardised (theta, phi, E) of rows (E, theta, phi, class), in FP32 like the kernels."""
    r = np.asarray(rows, dtype=np.float32)
    mean = np.asarray(mean, dtype=np.float32)
    inv = (np.float32(1.0) / np.asarray(std, dtype=np.float32)).astype(np.float32)
    x = np.stack([(r[:, 1] - mean[0]) * inv[0], (r[:, 2] - mean[1]) * inv[1], (r[:, 0] - mean[2]) * inv[2]], axis=1)
    return x.astype(np.float32).astype(np.float64)


def forward(params, rows, mean, std, n_classes, bf16_points=True):
    """Softmax probabilities [n][n_classes] and the cache for backward."""
    q = bf16 if bf16_points else (lambda v: np.asarray(v, dtype=np.float64))
    w = unpack(params)
    x = features(rows, mean, std)
    z1 = x @ w["W1"].T + w["b1"]
    h1 = q(np.maximum(z1, 0.0))
    z2 = h1 @ q(w["W2"]).T + w["b2"]
    h2 = q(np.maximum(z2, 0.0))
    z3 = h2 @ q(w["W3"]).T + w["b3"]
    h3 = q(np.maximum(z3, 0.0))
    logits = (h3 @ q(w["W4"]).T + w["b4"])[:, :n_classes]
    logits = logits - logits.max(axis=1, keepdims=True)
    e = np.exp(logits)
    p = e / e.sum(axis=1, keepdims=True)
    return p, dict(x=x, h1=h1, h2=h2, h3=h3, w=w, q=q)


def loss_and_grad(params, rows, mean, std, n_classes, bf16_points=True):
    """Mean cross-entropy and its gradient (packed like the parameters)."""
    rows = np.asarray(rows)
    n = len(rows)
    y = np.asarray(rows[:, 3], dtype=np.int64)
    p, c = forward(params, rows, mean, std, n_classes, bf16_points)
    q, w = c["q"], c["w"]
    loss = float(-np.log(np.maximum(p[np.arange(n), y], 1e-30)).mean())
    dl = p.copy()
    dl[np.arange(n), y] -= 1.0
    dl = np.pad(dl / n, ((0, 0), (0, OUT_PAD - n_classes)))
    dl = q(dl)
    g = {"W4": dl.T @ c["h3"], "b4": dl.sum(axis=0)}
    d = q((dl @ q(w["W4"])) * (c["h3"] > 0))
    g["W3"], g["b3"] = d.T @ c["h2"], d.sum(axis=0)
    d = q((d @ q(w["W3"])) * (c["h2"] > 0))
    g["W2"], g["b2"] = d.T @ c["h1"], d.sum(axis=0)
    d = q((d @ q(w["W2"])) * (c["h1"] > 0))
    g["W1"], g["b1"] = d.T @ c["x"], d.sum(axis=0)
    return loss, pack(g)


def arf_weights(p, russian_roulette):
    """Window weights of the network outputs: class 0 re-weighted by the
    Russian-roulette factor of the training rows, renormalised; columns 1.. = windows."""
    p = np.asarray(p, dtype=np.float64).copy()
    p[:, 0] *= russian_roulette
    return p / p.sum(axis=1, keepdims=True)
