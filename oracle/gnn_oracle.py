"""CPU oracle of the learned-start network -- TEST INFRASTRUCTURE ONLY.

FP64 numpy restatement of the bipartite row / column message-passing network
behind SK_START_LEARNED (3 layers, hidden width 64): forward pass, loss and the
analytic gradient w.r.t. every parameter, in the device code's parameter layout.
The device kernels compute with BF16 copies of the weights; `forward(...,
bf16=True)` rounds the FP32 master weights the same way (round to nearest
even) so that device and oracle evaluate the same function. Only tests/ use
this module, to check the device forward pass and gradients.

The network has no counterpart in the reference; its definition:
  column features f_c = (c_j, log(1 + nnz_j), ||A_.j||_2), row features
  f_r = (b_i, log(1 + nnz_i), ||A_i.||_2);
  h_c = relu(E_c f_c + e_c), h_r = relu(E_r f_r + e_r);
  per layer: m_r = deg_i^-1 A h_c; h_r = relu(W_rr h_r + W_rm m_r + b_r);
             m_c = deg_j^-1 A^T h_r; h_c = relu(W_cc h_c + W_cm m_c + b_c);
  outputs (log x, log s) = H_c h_c + o_c, y = H_r h_r + o_r;
  loss = (1/2n) sum_j [(log x_j - t_j)^2 + (log s_j - u_j)^2] + (1/m) sum_i (y_i - w_i)^2,
  log targets clipped to [-30, 30].
"""
import numpy as np
import scipy.sparse as sp

H = 64
L = 3


def layout():
    """name -> (offset, shape), in the device order."""
    out, o = {}, 0

    def add(name, shape):
        nonlocal o
        out[name] = (o, shape)
        o += int(np.prod(shape))

    add("Ec", (H, 3)); add("ec", (H,)); add("Er", (H, 3)); add("er", (H,))
    for l in range(L):
        add("Wrr%d" % l, (H, H)); add("Wrm%d" % l, (H, H)); add("br%d" % l, (H,))
        add("Wcc%d" % l, (H, H)); add("Wcm%d" % l, (H, H)); add("bc%d" % l, (H,))
    add("Hc", (2, H)); add("oc", (2,)); add("Hr", (1, H)); add("or", (1,))
    return out, o


def bf16_round(w):
    """FP32 -> BF16 -> FP64, round to nearest even (non-finite values kept)."""
    u = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    fin = (u & 0x7F800000) != 0x7F800000
    r = np.where(fin, u + 0x7FFF + ((u >> 16) & 1), u)
    r = ((r >> 16) << 16).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(params, bf16=True):
    lay, total = layout()
    p = np.asarray(params)
    assert p.size == total
    w = bf16_round(p.astype(np.float32)) if bf16 else p.astype(np.float64)
    return {k: w[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}


def pack_grad(g):
    lay, total = layout()
    out = np.zeros(total)
    for k, (o, s) in lay.items():
        out[o:o + int(np.prod(s))] = g[k].ravel()
    return out


def _relu(x):
    return np.maximum(x, 0.0)


def forward(params, m, n, rp, ci, vals, b, c, targets=None, bf16=True):
    """Returns (logx, logs, y, loss or None, cache)."""
    W = unpack(params, bf16)
    A = sp.csr_matrix((np.asarray(vals, float), np.asarray(ci), np.asarray(rp)), shape=(m, n))
    At = A.T.tocsr()
    deg_r = np.diff(A.indptr).astype(float)
    deg_c = np.diff(At.indptr).astype(float)
    fr = np.stack([np.asarray(b, float), np.log1p(deg_r), np.sqrt(np.asarray(A.multiply(A).sum(1)).ravel())], 1)
    fc = np.stack([np.asarray(c, float), np.log1p(deg_c), np.sqrt(np.asarray(A.multiply(A).sum(0)).ravel())], 1)
    ir = 1.0 / np.maximum(deg_r, 1.0)
    ic = 1.0 / np.maximum(deg_c, 1.0)
    hc = [_relu(fc @ W["Ec"].T + W["ec"])]
    hr = [_relu(fr @ W["Er"].T + W["er"])]
    mr, mc = [], []
    for l in range(L):
        mr.append(ir[:, None] * (A @ hc[l]))
        hr.append(_relu(hr[l] @ W["Wrr%d" % l].T + mr[l] @ W["Wrm%d" % l].T + W["br%d" % l]))
        mc.append(ic[:, None] * (At @ hr[l + 1]))
        hc.append(_relu(hc[l] @ W["Wcc%d" % l].T + mc[l] @ W["Wcm%d" % l].T + W["bc%d" % l]))
    oc = hc[L] @ W["Hc"].T + W["oc"]
    orr = hr[L] @ W["Hr"].T + W["or"]
    cache = dict(W=W, A=A, At=At, fr=fr, fc=fc, ir=ir, ic=ic, hc=hc, hr=hr, mr=mr, mc=mc, m=m, n=n)
    loss = None
    if targets is not None:
        tx, ts, ty = (np.asarray(t, float) for t in targets)
        ex = oc[:, 0] - np.clip(tx, -30, 30)
        es = oc[:, 1] - np.clip(ts, -30, 30)
        ey = orr[:, 0] - ty
        loss = (np.sum(ex * ex) + np.sum(es * es)) / (2 * n) + np.sum(ey * ey) / m
        cache["doc"] = np.stack([ex, es], 1) / n
        cache["dor"] = (2.0 / m) * ey[:, None]
    return oc[:, 0].copy(), oc[:, 1].copy(), orr[:, 0].copy(), loss, cache


def backward(cache):
    """Gradient of the loss of the last forward() w.r.t. every parameter (device layout)."""
    W, A, At = cache["W"], cache["A"], cache["At"]
    hc, hr, mr, mc, ir, ic = cache["hc"], cache["hr"], cache["mr"], cache["mc"], cache["ir"], cache["ic"]
    g = {}
    doc, dor = cache["doc"], cache["dor"]
    g["Hc"] = doc.T @ hc[L]; g["oc"] = doc.sum(0)
    g["Hr"] = dor.T @ hr[L]; g["or"] = dor.sum(0)
    dhc = doc @ W["Hc"]
    dhr = dor @ W["Hr"]
    for l in range(L - 1, -1, -1):
        gc = dhc * (hc[l + 1] > 0)
        g["Wcc%d" % l] = gc.T @ hc[l]; g["Wcm%d" % l] = gc.T @ mc[l]; g["bc%d" % l] = gc.sum(0)
        dhc_new = gc @ W["Wcc%d" % l]
        dmc = gc @ W["Wcm%d" % l]
        dhr = dhr + A @ (ic[:, None] * dmc)
        gr = dhr * (hr[l + 1] > 0)
        g["Wrr%d" % l] = gr.T @ hr[l]; g["Wrm%d" % l] = gr.T @ mr[l]; g["br%d" % l] = gr.sum(0)
        dhr_new = gr @ W["Wrr%d" % l]
        dmr = gr @ W["Wrm%d" % l]
        dhc_new = dhc_new + At @ (ir[:, None] * dmr)
        dhc, dhr = dhc_new, dhr_new
    gc = dhc * (hc[0] > 0)
    g["Ec"] = gc.T @ cache["fc"]; g["ec"] = gc.sum(0)
    gr = dhr * (hr[0] > 0)
    g["Er"] = gr.T @ cache["fr"]; g["er"] = gr.sum(0)
    return pack_grad(g)


def glorot_params(seed):
    """Random parameters for tests (not the device initialiser)."""
    rng = np.random.default_rng(seed)
    lay, total = layout()
    p = np.zeros(total, dtype=np.float32)
    for k, (o, s) in lay.items():
        if len(s) == 2:
            lim = np.sqrt(6.0 / (s[0] + s[1]))
            p[o:o + s[0] * s[1]] = rng.uniform(-lim, lim, s[0] * s[1])
        else:
            p[o:o + s[0]] = rng.uniform(0.0, 0.05, s[0])
    return p
