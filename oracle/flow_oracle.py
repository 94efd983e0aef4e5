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
