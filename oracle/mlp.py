"""Oracle (test infrastructure only): FP64 numpy restatement of the learned smoother's
element-local MLP (896 -> 256 -> 256 -> 256 -> 512, tanh-form GELU after the hidden
layers), its backward pass and one Adam step. The network has no counterpart in the
reference; this restatement is the checker for the CUDA forward/backward/Adam kernels.
"""
import numpy as np

DIMS = (896, 256, 256, 256, 512)
C = np.sqrt(2.0 / np.pi)


def param_count():
    return sum(DIMS[l] * DIMS[l + 1] + DIMS[l + 1] for l in range(4))


def unpack(theta):
    """Views (W_l, b_l) of the flat parameter vector (W row-major in x out)."""
    out, off = [], 0
    for l in range(4):
        n = DIMS[l] * DIMS[l + 1]
        W = theta[off:off + n].reshape(DIMS[l], DIMS[l + 1])
        off += n
        b = theta[off:off + DIMS[l + 1]]
        off += DIMS[l + 1]
        out.append((W, b))
    return out


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(C * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(C * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * C * (1 + 3 * 0.044715 * z * z)


def forward(theta, X):
    layers = unpack(np.asarray(theta, dtype=np.float64))
    a = np.asarray(X, dtype=np.float64)
    cache = [a]
    for l, (W, b) in enumerate(layers):
        z = a @ W + b
        if l < 3:
            cache.append(z)
            a = gelu(z)
            cache.append(a)
        else:
            a = z
    return a, cache


def backward(theta, X, dY):
    """Gradient of sum(dY * Y) with respect to the flat parameter vector."""
    layers = unpack(np.asarray(theta, dtype=np.float64))
    _, cache = forward(theta, X)
    acts = [cache[0], cache[2], cache[4], cache[6]]      # layer inputs
    pre = [cache[1], cache[3], cache[5]]                  # hidden pre-activations
    grads = [None] * 4
    d = np.asarray(dY, dtype=np.float64)
    for l in range(3, -1, -1):
        W, _ = layers[l]
        grads[l] = (acts[l].T @ d, d.sum(axis=0))
        if l == 0:
            break
        d = (d @ W.T) * gelu_grad(pre[l - 1])
    return np.concatenate([np.concatenate([g[0].ravel(), g[1]]) for g in grads])


def adam(w, g, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    w = w - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return w, m, v


def glorot(seed=0):
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(4):
        a = np.sqrt(6.0 / (DIMS[l] + DIMS[l + 1]))
        parts.append(rng.uniform(-a, a, DIMS[l] * DIMS[l + 1]))
        parts.append(rng.uniform(-0.1, 0.1, DIMS[l + 1]))
    return np.concatenate(parts)
