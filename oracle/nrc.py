"""FP64 numpy restatement of the neural radiance cache -- TEST INFRASTRUCTURE ONLY.

Restates the network the reference trains through tiny-cuda-nn (crates/akari_integrator/src/
nrc_pt.rs:1159-1352; crates/akari_cpp_ext/cpp_ext/akari_tcnn.cu:42-168) as configured in
include/sty_gb300.h: frequency encoding, ReLU MLP of width 64 without biases, linear output,
relative-L2 loss (prediction treated as constant in the denominator), Adam with exponential
learning-rate decay, debiased EMA of the weights. tiny-cuda-nn itself (git submodule, not vendored)
is absent: its published definitions of these components are what is restated.

`bf16=True` emulates the tensor-core path exactly up to FP32 accumulation order: weights and each
layer's input activations are rounded to bfloat16 (round to nearest even), products accumulate in
FP64 here (FP32 in TMEM on the GPU). In the gradient the loss gradient and each layer's
pre-activation gradient are rounded to bfloat16 before they enter a product, and the ReLU mask is
taken from the rounded activation.
"""
from __future__ import annotations

import numpy as np

W = 64


def fp16_round(x: np.ndarray) -> np.ndarray:
    """Round values to FP32 and then to the nearest IEEE half (ties to even), as float64: the GPU's
    cvt.rn.f16.f32 of an FP32 value."""
    return np.asarray(x, dtype=np.float32).astype(np.float16).astype(np.float64)


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float values to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32).copy()
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def encode(x: np.ndarray, freqs) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    cols = []
    for d, f in enumerate(freqs[: x.shape[1]]):
        for k in range(int(f)):
            a = np.pi * x[:, d] * (2.0 ** k)
            cols += [np.sin(a), np.cos(a)]
    enc = np.zeros((x.shape[0], W))
    if cols:
        enc[:, : len(cols)] = np.stack(cols, 1)
    return enc


def unflatten(params: np.ndarray, layers: int, out_dims: int):
    p = np.asarray(params, dtype=np.float64)
    mats = [p[l * W * W:(l + 1) * W * W].reshape(W, W) for l in range(layers)]
    mats.append(p[layers * W * W: layers * W * W + out_dims * W].reshape(out_dims, W))
    return mats


def forward(params, x, freqs, layers, out_dims, bf16=False):
    mats = unflatten(params, layers, out_dims)
    if bf16:
        mats = [bf16_round(m) for m in mats]
    h = encode(x, freqs)
    acts = [h]
    for l in range(layers):
        hin = bf16_round(h) if bf16 else h
        h = np.maximum(hin @ mats[l].T, 0.0)
        acts.append(h)
    hin = bf16_round(h) if bf16 else h
    return hin @ mats[layers].T, acts


def loss_and_grad(params, x, target, freqs, layers, out_dims, bf16=False):
    mats = unflatten(params, layers, out_dims)
    pred, acts = forward(params, x, freqs, layers, out_dims, bf16=bf16)
    rnd = bf16_round if bf16 else (lambda a: a)
    if bf16:
        mats = [bf16_round(m) for m in mats]
        acts = [bf16_round(a) for a in acts]
    B, C = pred.shape
    den = pred * pred + 0.01
    loss = float(((pred - target) ** 2 / den).mean())
    g = rnd(2.0 * (pred - target) / den / (B * C))
    grads = [None] * (layers + 1)
    grads[layers] = g.T @ acts[layers]
    dh = g @ mats[layers]
    for l in range(layers - 1, -1, -1):
        dp = rnd(dh * (acts[l + 1] > 0))
        grads[l] = dp.T @ acts[l]
        dh = dp @ mats[l]
    flat = np.concatenate([gm.reshape(-1) for gm in grads])
    return loss, flat


def adam(params, m, v, grad, step, lr, b1, b2, eps):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    params = params - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return params, m, v
