"""CPU restatement of the coupling-flow loss and gradient -- TEST
INFRASTRUCTURE ONLY (checks lensed_gb300/csrc/lg_flow.cu).

Same parameter layout as the library: for each coupling layer l and each
dense layer k (hidden layers then the output layer), a row-major weight
matrix [k_in x k_out] followed by the bias [k_out].  Layer l conditions on
A = [0, h) (even l) or [h, d) (odd l), h = d // 2, and transforms the other
half: z_B = u_B exp(s) + t, s = c tanh(s_raw / c), c = 5.  Loss = mean over
samples of 0.5 |z|^2 - sum s (constants dropped).  Float64 throughout.
"""
import numpy as np

CLAMP = 5.0


def layout(d, layers, width, hidden):
    h = d // 2
    out, off = [], 0
    for l in range(layers):
        da = h if l % 2 == 0 else d - h
        db = d - da
        dims = [da] + [width] * hidden + [2 * db]
        dense = []
        for k in range(hidden + 1):
            kin, kout = dims[k], dims[k + 1]
            dense.append((off, kin, kout, off + kin * kout))
            off += kin * kout + kout
        out.append((da, db, 0 if l % 2 == 0 else h, h if l % 2 == 0 else 0, dense))
    return out, off


def loss_grad(params, x, d, layers, width, hidden):
    L, n = layout(d, layers, width, hidden)
    p = np.asarray(params, np.float64)
    M = x.shape[0]
    grad = np.zeros_like(p)
    us, caches = [np.asarray(x, np.float64)], []
    logdet = np.zeros(M)
    for (da, db, a0, b0, dense) in L:
        u = us[-1]
        inp = u[:, a0:a0 + da]
        acts = [inp]
        for k, (w0, kin, kout, b) in enumerate(dense):
            W = p[w0:w0 + kin * kout].reshape(kin, kout)
            z = acts[-1] @ W + p[b:b + kout]
            acts.append(np.maximum(z, 0) if k < len(dense) - 1 else z)
        o = acts[-1]
        sr, t = o[:, :db], o[:, db:]
        s = CLAMP * np.tanh(sr / CLAMP)
        v = u.copy()
        v[:, b0:b0 + db] = u[:, b0:b0 + db] * np.exp(s) + t
        logdet += s.sum(1)
        caches.append((acts, sr, s))
        us.append(v)
    z = us[-1]
    loss = np.mean(0.5 * np.sum(z * z, 1) - logdet)
    dv = z / M
    for li in range(len(L) - 1, -1, -1):
        da, db, a0, b0, dense = L[li]
        acts, sr, s = caches[li]
        u = us[li]
        g = dv[:, b0:b0 + db]
        es = np.exp(s)
        ds = g * u[:, b0:b0 + db] * es - 1.0 / M
        th = np.tanh(sr / CLAMP)
        dout = np.concatenate([ds * (1 - th * th), g], axis=1)
        du = dv.copy()
        du[:, b0:b0 + db] = g * es
        dcur = dout
        for k in range(len(dense) - 1, -1, -1):
            w0, kin, kout, b = dense[k]
            W = p[w0:w0 + kin * kout].reshape(kin, kout)
            grad[w0:w0 + kin * kout] = (acts[k].T @ dcur).ravel()
            grad[b:b + kout] = dcur.sum(0)
            dprev = dcur @ W.T
            if k > 0:
                dprev = dprev * (acts[k] > 0)
            dcur = dprev
        du[:, a0:a0 + da] += dcur
        dv = du
    return loss, grad


def bf16(a):
    """Round float64 values to bfloat16 (through float32, round to nearest
    even), returned as float64."""
    f = np.asarray(a, np.float64).astype(np.float32)
    bits = f.view(np.uint32).astype(np.uint64)
    bits = (bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000
    return bits.astype(np.uint32).view(np.float32).astype(np.float64)


def loss_grad_tc(params, x, d, layers, width, hidden):
    """loss_grad with the rounding points of the tensor-core training step
    (lg_flow_step_tc): weights, conditioner input and hidden activations in
    bfloat16 (forward), the output-layer gradient dO and the masked hidden
    gradients dY rounded to bfloat16 before they enter the products;
    dense-layer bias gradients summed from the rounded dY, the output bias
    gradient from the unrounded dO.  Float64 arithmetic otherwise."""
    L, n = layout(d, layers, width, hidden)
    p = np.asarray(params, np.float64)
    M = x.shape[0]
    grad = np.zeros_like(p)
    us, caches = [np.asarray(x, np.float64)], []
    logdet = np.zeros(M)
    for (da, db, a0, b0, dense) in L:
        u = us[-1]
        acts = [bf16(u[:, a0:a0 + da])]
        for k, (w0, kin, kout, b) in enumerate(dense):
            W = bf16(p[w0:w0 + kin * kout].reshape(kin, kout))
            z = acts[-1] @ W + p[b:b + kout]
            acts.append(bf16(np.maximum(z, 0)) if k < len(dense) - 1 else z)
        o = acts[-1]
        sr, t = o[:, :db], o[:, db:]
        s = CLAMP * np.tanh(sr / CLAMP)
        v = u.copy()
        v[:, b0:b0 + db] = u[:, b0:b0 + db] * np.exp(s) + t
        logdet += s.sum(1)
        caches.append((acts, sr, s))
        us.append(v)
    z = us[-1]
    loss = np.mean(0.5 * np.sum(z * z, 1) - logdet)
    dv = z / M
    for li in range(len(L) - 1, -1, -1):
        da, db, a0, b0, dense = L[li]
        acts, sr, s = caches[li]
        u = us[li]
        g = dv[:, b0:b0 + db]
        es = np.exp(s)
        ds = g * u[:, b0:b0 + db] * es - 1.0 / M
        th = np.tanh(sr / CLAMP)
        dout = np.concatenate([ds * (1 - th * th), g], axis=1)
        du = dv.copy()
        du[:, b0:b0 + db] = g * es
        w0, kin, kout, b = dense[-1]
        grad[b:b + kout] = dout.sum(0)
        dcur = bf16(dout)
        for k in range(len(dense) - 1, -1, -1):
            w0, kin, kout, b = dense[k]
            W = bf16(p[w0:w0 + kin * kout].reshape(kin, kout))
            grad[w0:w0 + kin * kout] = (acts[k].T @ dcur).ravel()
            if k < len(dense) - 1:
                grad[b:b + kout] = dcur.sum(0)
            dprev = dcur @ W.T
            if k > 0:
                dprev = bf16(dprev * (acts[k] > 0))
            dcur = dprev
        du[:, a0:a0 + da] += dcur
        dv = du
    return loss, grad


def inverse(params, z, d, layers, width, hidden, mode="fp32"):
    """Inverse flow z -> u and log|det du/dz| in float64, with the rounding
    points of the library's kernels: mode "fp32" none, "bf16" hidden
    activations rounded to bfloat16 (FP32-weight kernel), "tc" also the
    weights and the conditioner input (tensor-core kernel)."""
    L, n = layout(d, layers, width, hidden)
    p = np.asarray(params, np.float64)
    cur = np.array(z, np.float64)
    ld = np.zeros(cur.shape[0])
    for (da, db, a0, b0, dense) in reversed(L):
        x = cur[:, a0:a0 + da]
        if mode == "tc":
            x = bf16(x)
        for k, (w0, kin, kout, b) in enumerate(dense):
            W = p[w0:w0 + kin * kout].reshape(kin, kout)
            if mode == "tc":
                W = bf16(W)
            x = x @ W + p[b:b + kout]
            if k < len(dense) - 1:
                x = np.maximum(x, 0)
                if mode in ("bf16", "tc"):
                    x = bf16(x)
        sr, t = x[:, :db], x[:, db:]
        s = CLAMP * np.tanh(sr / CLAMP)
        cur[:, b0:b0 + db] = (cur[:, b0:b0 + db] - t) * np.exp(-s)
        ld -= s.sum(1)
    return cur, ld
