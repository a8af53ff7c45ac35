"""NumPy FP64 restatement of the MGFM seed surrogate (12-64-64-64-2, tanh) for
the device-kernel tests: forward pass, loss and backpropagated gradients.

The parameter vector follows the library's layout
    W1[64][12] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[2][64] b4[2]
    mean_x[12] std_x[12] mean_y[2] std_y[2]
With bf16=True the weight matrices (not the biases) are rounded to bfloat16
(round to nearest even) before use; the gradient is the straight-through one
(the rounding is treated as the identity), which is what the device computes.
"""
import numpy as np

NI, NH, NO = 12, 64, 2
SHAPES = [(NH, NI), (NH, NH), (NH, NH), (NO, NH)]
NPARAM = sum(a * b + a for a, b in SHAPES)


def bf16_round(w):
    """float32 -> bfloat16 (round to nearest, ties to even) -> float32."""
    u = np.ascontiguousarray(w, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p, bf16=False):
    p = np.asarray(p)
    layers, o = [], 0
    for a, b in SHAPES:
        W = p[o:o + a * b].reshape(a, b)
        if bf16:
            W = bf16_round(W.astype(np.float32))
        o += a * b
        layers.append((W.astype(np.float64), p[o:o + a].astype(np.float64)))
        o += a
    nrm = p[NPARAM:].astype(np.float64)
    mx, sx, my, sy = nrm[:NI], nrm[NI:2 * NI], nrm[2 * NI:2 * NI + NO], nrm[2 * NI + NO:]
    return layers, (mx, sx, my, sy)


def forward(p, X, bf16=False):
    """Normalised outputs Y [n, 2] and the activations (input, h1, h2, h3)."""
    layers, (mx, sx, _, _) = unpack(p, bf16)
    a = (np.asarray(X, np.float64) - mx) / sx
    acts = [a]
    for W, b in layers[:-1]:
        a = np.tanh(a @ W.T + b)
        acts.append(a)
    W, b = layers[-1]
    return a @ W.T + b, acts


def loss_grad(p, X, T, bf16=False):
    """Loss mean((Y - normalise(T))^2) over n x 2 and its gradient (NPARAM)."""
    layers, (_, _, my, sy) = unpack(p, bf16)
    Y, acts = forward(p, X, bf16)
    Tn = (np.asarray(T, np.float64) - my) / sy
    d = Y - Tn
    m = d.size
    loss = float((d * d).sum() / m)
    dz = 2.0 * d / m
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        W, _ = layers[li]
        a_in = acts[li]
        grads.append((dz.T @ a_in, dz.sum(0)))
        if li > 0:
            dz = (dz @ W) * (1.0 - a_in * a_in)
    g = []
    for gW, gb in reversed(grads):
        g.append(gW.ravel())
        g.append(gb)
    return loss, np.concatenate(g)


def forward_bf16_act(p, X):
    """Forward pass with BF16 weights and BF16 activations (the tensor-core
    path): normalised inputs and each hidden layer's tanh output are rounded to
    BF16 before the next layer; sums and biases in FP64."""
    layers, (mx, sx, _, _) = unpack(p, bf16=True)
    a = bf16_round(((np.asarray(X, np.float64) - mx) / sx).astype(np.float32)).astype(np.float64)
    for W, b in layers[:-1]:
        a = bf16_round(np.tanh(a @ W.T + b).astype(np.float32)).astype(np.float64)
    W, b = layers[-1]
    return a @ W.T + b
