"""TEST ORACLE for the path-guiding network: FP64 numpy restatement of the
hash-grid encoding, MLP, 8-lobe vMF mixture head and the gradient of the
training loss  L = -sum_j c_j log q(w_j | x_j) / sum_j c_j.  The network has
no counterpart in the reference; this oracle is written from the
mathematics and is used only by tests/ to check the GPU forward pass and
gradients.  Parameter layout follows include/gbrt.h (gbrt_guide_get_params).
"""
import math

import numpy as np

LEVELS, FEAT, IN, HID, LOBES = 16, 2, 32, 64, 8
OUT = 5 * LOBES
KMIN, KMAX = 0.05, 2000.0
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * IN
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + OUT * HID
N_MLP = OFF_B3 + OUT


class Grid:
    def __init__(self, bound, log2_table=19, base_res=16.0, max_res=2048.0):
        b = np.asarray(bound, np.float32)
        self.lo = b[:3].astype(np.float64)
        ext = (b[3:] - b[:3]).astype(np.float32)
        self.inv_ext = np.where(ext > 0, np.float32(1.0) / np.where(ext > 0, ext, 1), 0).astype(np.float32).astype(np.float64)
        self.log2_table = log2_table
        g = math.exp((math.log(max_res) - math.log(base_res)) / (LEVELS - 1))
        self.res = [float(np.floor(np.float32(base_res * g ** l))) for l in range(LEVELS)]
        self.dense = [((r + 1.0) ** 3) <= float(1 << log2_table) for r in self.res]

    def index(self, level, ix, iy, iz):
        T = 1 << self.log2_table
        if self.dense[level]:
            r = int(self.res[level]) + 1
            return (ix + r * (iy + r * iz)) & (T - 1)
        return (ix ^ ((iy * 2654435761) & 0xFFFFFFFF) ^ ((iz * 805459861) & 0xFFFFFFFF)) & (T - 1)

    def encode(self, table, p):
        """table: [LEVELS, T, FEAT]; returns (e[32], corners list of (level, idx, w))."""
        x = np.clip((np.asarray(p, np.float64) - self.lo) * self.inv_ext, 0.0, 1.0)
        e = np.zeros(IN)
        corners = []
        for l in range(LEVELS):
            r = self.res[l]
            s = x * r
            fl = np.minimum(np.floor(s), r - 1.0)
            ix = fl.astype(np.int64)
            fx = s - fl
            for c in range(8):
                d = (c & 1, (c >> 1) & 1, (c >> 2) & 1)
                w = np.prod([fx[a] if d[a] else 1.0 - fx[a] for a in range(3)])
                idx = self.index(l, int(ix[0] + d[0]), int(ix[1] + d[1]), int(ix[2] + d[2]))
                e[2 * l:2 * l + 2] += w * table[l, idx]
                corners.append((l, idx, w))
        return e, corners


def softplus(x):
    return x if x > 20 else math.log1p(math.exp(x))


def mlp_forward(mlp, e):
    W1 = mlp[OFF_W1:OFF_B1].reshape(HID, IN); b1 = mlp[OFF_B1:OFF_W2]
    W2 = mlp[OFF_W2:OFF_B2].reshape(HID, HID); b2 = mlp[OFF_B2:OFF_W3]
    W3 = mlp[OFF_W3:OFF_B3].reshape(OUT, HID); b3 = mlp[OFF_B3:N_MLP]
    a1 = W1 @ e + b1; h1 = np.maximum(a1, 0)
    a2 = W2 @ h1 + b2; h2 = np.maximum(a2, 0)
    o = W3 @ h2 + b3
    return h1, h2, o


def lobes(o):
    out = np.zeros(OUT)
    logits = o[4::5]
    w = np.exp(logits - logits.max()); w /= w.sum()
    for k in range(LOBES):
        m = o[5 * k:5 * k + 3]
        n = np.linalg.norm(m)
        out[5 * k:5 * k + 3] = m / n if n > 1e-20 else (0, 0, 1)
        out[5 * k + 3] = min(softplus(o[5 * k + 3]) + KMIN, KMAX)
        out[5 * k + 4] = w[k]
    return out


def vmf_log_pdf(mu, kap, w):
    return math.log(kap) - math.log(2 * math.pi) - math.log(-math.expm1(-2 * kap)) + kap * (float(np.dot(mu, w)) - 1.0)


def mixture_pdf(lob, w):
    return sum(lob[5 * k + 4] * math.exp(vmf_log_pdf(lob[5 * k:5 * k + 3], lob[5 * k + 3], w)) for k in range(LOBES))


def loss_and_grads(grid, mlp, table, records):
    """records: [n, 8] (pos xyz, dir xyz, c, pad).  Returns (loss, dmlp, dtable)."""
    mlp = np.asarray(mlp, np.float64)
    table = np.asarray(table, np.float64)
    W1 = mlp[OFF_W1:OFF_B1].reshape(HID, IN)
    W2 = mlp[OFF_W2:OFF_B2].reshape(HID, HID)
    W3 = mlp[OFF_W3:OFF_B3].reshape(OUT, HID)
    dmlp = np.zeros(N_MLP)
    dtable = np.zeros_like(table)
    csum = float(np.sum(records[:, 6]))
    loss = 0.0
    for r in records:
        p, w, c = r[:3], r[3:6].astype(np.float64), float(r[6]) / csum
        e, corners = grid.encode(table, p)
        h1, h2, o = mlp_forward(mlp, e)
        lob = lobes(o)
        logf = np.array([math.log(lob[5 * k + 4]) + vmf_log_pdf(lob[5 * k:5 * k + 3], lob[5 * k + 3], w) for k in range(LOBES)])
        lmax = logf.max()
        logq = lmax + math.log(np.exp(logf - lmax).sum())
        loss += -c * logq
        d3 = np.zeros(OUT)
        for k in range(LOBES):
            rk = math.exp(logf[k] - logq)
            wk, kap = lob[5 * k + 4], lob[5 * k + 3]
            mu = lob[5 * k:5 * k + 3]
            mw = float(np.dot(mu, w))
            d3[5 * k + 4] = c * (wk - rk)
            e2 = math.exp(-2 * kap)
            dl = 1.0 / kap - 2 * e2 / (1 - e2) + (mw - 1.0)
            a = o[5 * k + 3]
            dk = 1.0 / (1.0 + math.exp(-a)) if softplus(a) + KMIN < KMAX else 0.0
            d3[5 * k + 3] = -c * rk * dl * dk
            m = o[5 * k:5 * k + 3]
            ln = np.linalg.norm(m)
            if ln > 1e-20:
                d3[5 * k:5 * k + 3] = -c * rk * kap / ln * (w - mw * mu)
        d2 = (W3.T @ d3) * (h2 > 0)
        d1 = (W2.T @ d2) * (h1 > 0)
        de = W1.T @ d1
        dmlp[OFF_W3:OFF_B3] += np.outer(d3, h2).ravel(); dmlp[OFF_B3:N_MLP] += d3
        dmlp[OFF_W2:OFF_B2] += np.outer(d2, h1).ravel(); dmlp[OFF_B2:OFF_W3] += d2
        dmlp[OFF_W1:OFF_B1] += np.outer(d1, e).ravel(); dmlp[OFF_B1:OFF_W2] += d1
        for (l, idx, wc) in corners:
            dtable[l, idx] += wc * de[2 * l:2 * l + 2]
    return loss, dmlp, dtable
