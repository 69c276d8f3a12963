"""FP64 CPU restatement of the differentiable leaky-integrator rate network.

Test infrastructure only: the reference has no differentiable model, so this
is the checker for the GB300 forward pass and hand-written adjoint
(synaptogenesis_gb300/csrc/rate_adjoint.cu), and the CPU baseline the bench
times.  Parity against the reference is unpinned; the adjoint here is checked
against central finite differences of this same FP64 loss.

Model (per batch element, layers l = 0..L-1 of N = rows x cols neurons):
    I_0[t] = x[t];  I_l[t] = sum_k W_l[i, k] r_{l-1}[t-1][src(i, k)]
    v_l[t] = v_l[t-1] + (dt / tau_l) (-v_l[t-1] + I_l[t]),  r = sigmoid(v)
    y[t] = R r_{L-1}[t];  loss = mean over (t, b, o) of (y - target)^2
Convergent geometry: the reference's arborized window
(src/core/engine/kernel/synapse_kernel.h:384-421) with stride 1, spacing 1,
offset -field/2, no wrap (out-of-range sources skipped).
"""
import numpy as np
import scipy.sparse as sp


def conv_matrix(rows, cols, field, w):
    """Sparse N x N matrix C with C[i, src(i, k)] = w[i, k] (no wrap)."""
    h = field // 2
    N = rows * cols
    i = np.arange(N)
    ir, ic = i // cols, i % cols
    data, ri, ci = [], [], []
    for k in range(field * field):
        kr, kc = divmod(k, field)
        sr, sc = ir - h + kr, ic - h + kc
        ok = (sr >= 0) & (sr < rows) & (sc >= 0) & (sc < cols)
        ri.append(i[ok])
        ci.append((sr * cols + sc)[ok])
        data.append(w[ok, k])
    return sp.csr_matrix((np.concatenate(data), (np.concatenate(ri), np.concatenate(ci))),
                         shape=(N, N))


def conv_sources(rows, cols, field):
    """src[i, k] (or -1 where the source is out of range)."""
    h = field // 2
    N = rows * cols
    i = np.arange(N)
    ir, ic = i // cols, i % cols
    out = np.full((N, field * field), -1, np.int64)
    for k in range(field * field):
        kr, kc = divmod(k, field)
        sr, sc = ir - h + kr, ic - h + kc
        ok = (sr >= 0) & (sr < rows) & (sc >= 0) & (sc < cols)
        out[ok, k] = (sr * cols + sc)[ok]
    return out


def sigmoid(v):
    return 1.0 / (1.0 + np.exp(-v))


def forward(shape, x, w, R, tau, target):
    """Returns (loss, y, v, r, d): v, r [L][T+1][B][N], d [L][T][B][N]."""
    L, rows, cols, field = shape["layers"], shape["rows"], shape["cols"], shape["field"]
    T, B = shape["steps"], shape["batch"]
    dt = float(shape["dt"])
    N = rows * cols
    x = np.asarray(x, np.float64).reshape(T, B, N)
    w = np.asarray(w, np.float64).reshape(max(L - 1, 0), N, field * field)
    R = np.asarray(R, np.float64).reshape(-1, N)
    tau = np.asarray(tau, np.float64)
    target = np.asarray(target, np.float64).reshape(B, -1)
    C = [conv_matrix(rows, cols, field, w[l]) for l in range(L - 1)]
    a = dt / tau
    v = np.zeros((L, T + 1, B, N))
    r = np.zeros((L, T + 1, B, N))
    d = np.zeros((L, T, B, N))
    r[:, 0] = sigmoid(0.0)
    y = np.zeros((T, B, R.shape[0]))
    for t in range(1, T + 1):
        for l in range(L):
            I = x[t - 1] if l == 0 else (C[l - 1] @ r[l - 1, t - 1].T).T
            d[l, t - 1] = -v[l, t - 1] + I
            v[l, t] = v[l, t - 1] + a[l] * d[l, t - 1]
            r[l, t] = sigmoid(v[l, t])
        y[t - 1] = r[L - 1, t] @ R.T
    loss = np.mean((y - target[None]) ** 2)
    return loss, y, v, r, d


def adjoint(shape, x, w, R, tau, target, grad_loss=1.0):
    """Returns (loss, dw [L-1][N][K], dR [O][N], dtau [L], dx [T][B][N])."""
    L, rows, cols, field = shape["layers"], shape["rows"], shape["cols"], shape["field"]
    T, B = shape["steps"], shape["batch"]
    dt = float(shape["dt"])
    N, K = rows * cols, field * field
    loss, y, v, r, d = forward(shape, x, w, R, tau, target)
    w = np.asarray(w, np.float64).reshape(max(L - 1, 0), N, K)
    R = np.asarray(R, np.float64).reshape(-1, N)
    tau = np.asarray(tau, np.float64)
    target = np.asarray(target, np.float64).reshape(B, -1)
    O = R.shape[0]
    a = dt / tau
    C = [conv_matrix(rows, cols, field, w[l]) for l in range(L - 1)]
    src = conv_sources(rows, cols, field)
    valid = src >= 0
    srcc = np.where(valid, src, 0)
    scale = grad_loss * 2.0 / (T * B * O)
    lam_next = np.zeros((L, B, N))
    dw = np.zeros((max(L - 1, 0), N, K))
    dR = np.zeros((O, N))
    da = np.zeros(L)
    dx = np.zeros((T, B, N))
    for t in range(T, 0, -1):
        gy = scale * (y[t - 1] - target)
        lam = np.zeros((L, B, N))
        for l in range(L):
            if l == L - 1:
                g = gy @ R
            else:
                g = (C[l] .T @ (a[l + 1] * lam_next[l + 1]).T).T
            rr = r[l, t]
            lam[l] = rr * (1.0 - rr) * g + (1.0 - a[l]) * lam_next[l]
        for l in range(1, L):
            gathered = r[l - 1, t - 1][:, srcc]              # [B, N, K]
            dw[l - 1] += a[l] * np.einsum("bj,bjk->jk", lam[l], gathered) * valid
        dR += gy.T @ r[L - 1, t]
        da += np.einsum("lbn,lbn->l", lam, d[:, t - 1])
        dx[t - 1] = a[0] * lam[0]
        lam_next = lam
    dtau = da * (-dt / tau ** 2)
    return loss, dw, dR, dtau, dx


def finite_difference(shape, x, w, R, tau, target, which, index, h=1e-3):
    """Central difference of the FP64 loss in one parameter:
    which in {"w", "R", "tau"}, index a flat index into that array."""
    params = {"w": np.array(w, np.float64), "R": np.array(R, np.float64),
              "tau": np.array(tau, np.float64)}
    p = params[which].reshape(-1)
    base = p[index]
    p[index] = base + h
    lp = forward(shape, x, params["w"], params["R"], params["tau"], target)[0]
    p[index] = base - h
    lm = forward(shape, x, params["w"], params["R"], params["tau"], target)[0]
    p[index] = base
    return (lp - lm) / (2.0 * h)
