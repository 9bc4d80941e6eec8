"""FP64 numpy reference of the secular-predictor MLP -- TEST INFRASTRUCTURE.

Same parameter layout as the library (W1[NF][NH], b1, W2[NH][NH], b2, W3, b3,
W4[NH], b4), ReLU hidden layers, loss = mean((mlp((x - mu)/sd) - t)^2).  The
GPU gradient kernel is checked against :func:`loss_and_grad`.
"""
import numpy as np

NF, NH = 8, 64


def unpack(W):
    W = np.asarray(W, dtype=np.float64)
    o = 0
    out = []
    for shape in [(NF, NH), (NH,), (NH, NH), (NH,), (NH, NH), (NH,), (NH,), (1,)]:
        sz = int(np.prod(shape))
        out.append(W[o:o + sz].reshape(shape))
        o += sz
    assert o == W.size
    return out


def loss_and_grad(X, T, norm, W):
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(W)
    norm = np.asarray(norm, dtype=np.float64)
    x = (np.asarray(X, dtype=np.float64) - norm[:NF]) / norm[NF:]
    t = np.asarray(T, dtype=np.float64)
    n = len(t)
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0)
    z3 = h2 @ W3 + b3
    h3 = np.maximum(z3, 0)
    y = h3 @ W4 + b4[0]
    e = y - t
    loss = np.mean(e * e)
    dy = 2 * e / n
    gW4 = h3.T @ dy
    gb4 = np.array([dy.sum()])
    d3 = np.outer(dy, W4) * (z3 > 0)
    gW3 = h2.T @ d3
    gb3 = d3.sum(0)
    d2 = (d3 @ W3.T) * (z2 > 0)
    gW2 = h1.T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ W2.T) * (z1 > 0)
    gW1 = x.T @ d1
    gb1 = d1.sum(0)
    G = np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4)])
    return loss, G
