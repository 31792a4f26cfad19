"""FP64 numpy oracle of the learned emitter closure (test infrastructure only: the GPU library
never imports it).  The closure has no counterpart in the reference; this file defines its
arithmetic for the gradient and forward checks of the tensor-core implementation.

Network, per emitter and quantum step t (W = 32 window samples, H = 128 hidden, F = 256 width):
    x_t  = the last W samples of the field on the emitter's dipole axis (scaled), oldest first
    XH   = [x_t, h_{t-1}]                                    (W + H)
    G    = XH Wg^T + bg                                      (4H: r | z | nx | nh blocks)
           (the nx rows see only x, the nh rows only h: their other columns are masked to 0)
    r = sigmoid(G_r), z = sigmoid(G_z), n = tanh(G_nx + r * G_nh)
    h_t  = (1 - z) n + z h_{t-1}
    a1 = tanh(h_t W1^T + b1), a2 = tanh(a1 W2^T + b2), a3 = tanh(a2 W3^T + b3)
    y_t  = a3 w4 + b4                                        (the scaled dipole on the axis)
Loss: mean over emitters and steps t >= skip of (y_t - target_t)^2.

Parameter order of the flat vector (the library's order): Wg, bg, W1, b1, W2, b2, W3, b3, w4, b4.
"""
import numpy as np

W, H, F = 32, 128, 256
SHAPES = [("Wg", (4 * H, W + H)), ("bg", (4 * H,)), ("W1", (F, H)), ("b1", (F,)), ("W2", (F, F)), ("b2", (F,)),
          ("W3", (F, F)), ("b3", (F,)), ("w4", (F,)), ("b4", (1,))]


def n_params():
    return sum(int(np.prod(s)) for _, s in SHAPES)


def wg_mask():
    m = np.ones((4 * H, W + H))
    m[2 * H:3 * H, W:] = 0.0      # nx: input columns only
    m[3 * H:, :W] = 0.0           # nh: hidden columns only
    return m


def unpack(flat):
    out, o = {}, 0
    for name, shape in SHAPES:
        k = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + k], np.float64).reshape(shape)
        o += k
    return out


def pack(p):
    return np.concatenate([np.asarray(p[name], np.float64).ravel() for name, _ in SHAPES])


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def windows(e, T):
    """e: (B, T + W - 1) field samples -> x: (T, B, W), x_t = e[:, t : t + W]."""
    return np.stack([e[:, t:t + W] for t in range(T)], axis=0)


def forward(flat, e, T):
    """Returns y (T, B) and the activations the backward pass needs."""
    p = unpack(flat)
    Wg = p["Wg"] * wg_mask()
    B = e.shape[0]
    x = windows(e, T)
    h = np.zeros((B, H))
    cache = []
    ys = []
    for t in range(T):
        xh = np.concatenate([x[t], h], axis=1)
        g = xh @ Wg.T + p["bg"]
        r, z = sigmoid(g[:, :H]), sigmoid(g[:, H:2 * H])
        nx, nh = g[:, 2 * H:3 * H], g[:, 3 * H:]
        n = np.tanh(nx + r * nh)
        h_new = (1.0 - z) * n + z * h
        a1 = np.tanh(h_new @ p["W1"].T + p["b1"])
        a2 = np.tanh(a1 @ p["W2"].T + p["b2"])
        a3 = np.tanh(a2 @ p["W3"].T + p["b3"])
        y = a3 @ p["w4"] + p["b4"][0]
        cache.append((xh, r, z, n, nh, h, h_new, a1, a2, a3))
        ys.append(y)
        h = h_new
    return np.stack(ys, axis=0), cache


def loss_and_grad(flat, e, target, T, skip=0):
    """target: (T, B).  Mean squared error over t >= skip and its gradient (flat, FP64)."""
    p = unpack(flat)
    Wg = p["Wg"] * wg_mask()
    y, cache = forward(flat, e, T)
    B = e.shape[0]
    cnt = (T - skip) * B
    diff = y - target
    loss = float(np.sum(diff[skip:] ** 2) / cnt)
    g = {name: np.zeros(shape) for name, shape in SHAPES}
    dh_next = np.zeros((B, H))
    for t in reversed(range(T)):
        xh, r, z, n, nh, h_prev, h_new, a1, a2, a3 = cache[t]
        dy = (2.0 / cnt) * diff[t] if t >= skip else np.zeros(B)
        g["w4"] += a3.T @ dy
        g["b4"][0] += dy.sum()
        dz3 = np.outer(dy, p["w4"]) * (1.0 - a3 ** 2)
        g["W3"] += dz3.T @ a2
        g["b3"] += dz3.sum(0)
        dz2 = (dz3 @ p["W3"]) * (1.0 - a2 ** 2)
        g["W2"] += dz2.T @ a1
        g["b2"] += dz2.sum(0)
        dz1 = (dz2 @ p["W2"]) * (1.0 - a1 ** 2)
        g["W1"] += dz1.T @ h_new
        g["b1"] += dz1.sum(0)
        dh = dz1 @ p["W1"] + dh_next
        dn = dh * (1.0 - z)
        dzg = dh * (h_prev - n) * z * (1.0 - z)
        dpre_n = dn * (1.0 - n ** 2)
        drg = dpre_n * nh * r * (1.0 - r)
        dG = np.concatenate([drg, dzg, dpre_n, dpre_n * r], axis=1)
        g["Wg"] += (dG.T @ xh) * wg_mask()
        g["bg"] += dG.sum(0)
        dxh = dG @ Wg
        dh_next = dxh[:, W:] + dh * z
    return loss, pack(g)


def init_params(seed):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases (the update gate starts
    biased towards keeping the state: bg_z = 1)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, shape in SHAPES:
        if len(shape) == 2:
            p[name] = rng.uniform(-1, 1, shape) / np.sqrt(shape[1])
        elif name == "w4":
            p[name] = rng.uniform(-1, 1, shape) / np.sqrt(F)
        else:
            p[name] = np.zeros(shape)
    p["Wg"] = p["Wg"] * wg_mask()
    p["bg"][H:2 * H] = 1.0
    return pack(p)


def adam(flat, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return flat - lr * mh / (np.sqrt(vh) + eps), m, v
