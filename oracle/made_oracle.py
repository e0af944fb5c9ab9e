"""CPU restatement of the learned patch proposal (test infrastructure: the
checker of the CUDA kernels in uppasd_gb300/csrc/learned.cu; nothing in the
product imports it).

* MADE network over the 8 x 8 window (192 features, position-major xyz),
  three tanh layers, output eta = eta_scale * O (3 per patch spin, 48 of 64);
* the loss  L = -(1/R) sum_rows sum_s log vMF(x_s; eta_s)  and its gradient,
  in float64, either exact or emulating the GPU's bf16 rounding points
  (inputs, weights, hidden activations, dO and the backward activations);
* vMF log density and the exact energy change of a patch move from the
  simulation's neighbour lists (the terms of the reference's
  calculate_energy, MonteCarlo/montecarlo_common.f90:431-865: exchange, DMI,
  Zeeman), used to check the GPU's Metropolis-Hastings ratio.

The reference has no learned proposal; "parity" here is with this file's
float64 algebra, which the tests pin by finite differences.
"""
from __future__ import annotations

import numpy as np

N_FEAT, N_HID, N_OUT, N_SPIN = 192, 256, 64, 16


def round_bf16(x):
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((a >> 16) & 1) + np.uint32(0x7FFF)
    return (((a + r) >> 16) << 16).astype(np.uint32).view(np.float32).astype(np.float64)


def patch_group(py, px):
    return (py % 2) * 2 + (px % 2)


def feat_degree(f):
    pos = f // 3
    wy, wx = pos // 8, pos % 8
    if 2 <= wy < 6 and 2 <= wx < 6:
        return patch_group(wy - 2, wx - 2) + 1
    return 0


def masks():
    """MADE masks: hidden degree h % 4; outputs of group g see hidden degrees <= g."""
    din = np.array([feat_degree(f) for f in range(N_FEAT)])
    dh = np.arange(N_HID) % 4
    m1 = (din[None, :] <= dh[:, None]).astype(np.float64)
    m2 = (dh[None, :] <= dh[:, None]).astype(np.float64)
    m4 = np.zeros((N_OUT, N_HID))
    for o in range(48):
        s = o // 3
        m4[o] = (dh <= patch_group(s // 4, s % 4)).astype(np.float64)
    return [m1, m2, m2.copy(), m4]


def interior_positions():
    return np.array([(py + 2) * 8 + (px + 2) for py in range(4) for px in range(4)])


def patch_spins(X):
    """(R, 16, 3) patch spins from windows (R, 192)."""
    pos = interior_positions()
    idx = (pos[:, None] * 3 + np.arange(3)[None, :])
    return X[:, idx]


def log_vmf(eta, x):
    kap = np.linalg.norm(eta, axis=-1)
    dot = np.sum(eta * x, axis=-1)
    small = kap < 1e-8
    ks = np.where(small, 1.0, kap)
    val = dot + np.log(ks) - np.log(2 * np.pi) - np.log(-np.expm1(-2 * ks)) - ks
    return np.where(small, dot - np.log(4 * np.pi), val)


def unpack(vec):
    shapes = [(N_HID, N_FEAT), (N_HID, N_HID), (N_HID, N_HID), (N_OUT, N_HID)]
    ws, o = [], 0
    for s in shapes:
        ws.append(np.asarray(vec[o:o + s[0] * s[1]], dtype=np.float64).reshape(s))
        o += s[0] * s[1]
    bs = []
    for n in (N_HID, N_HID, N_HID, N_OUT):
        bs.append(np.asarray(vec[o:o + n], dtype=np.float64))
        o += n
    return ws, bs


def forward(vec, X, bf16=False):
    rb = round_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    ws, bs = unpack(vec)
    wb = [rb(w) for w in ws]
    h = rb(X)
    hs = [h]
    for l in range(3):
        h = rb(np.tanh(h @ wb[l].T + bs[l]))
        hs.append(h)
    O = h @ wb[3].T + bs[3]
    return O, hs, wb


def loss_grad(vec, X, eta_scale, bf16=False):
    """Loss and gradient in the parameter-vector layout."""
    rb = round_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    O, hs, wb = forward(vec, X, bf16)
    R = X.shape[0]
    x = patch_spins(hs[0])
    eta = eta_scale * O[:, :48].reshape(R, 16, 3)
    loss = -np.sum(log_vmf(eta, x)) / R
    kap = np.linalg.norm(eta, axis=-1, keepdims=True)
    a_over_k = np.where(kap < 1e-3, 1.0 / 3.0 - kap ** 2 / 45.0,
                        (1.0 / np.tanh(np.maximum(kap, 1e-300)) - 1.0 / np.maximum(kap, 1e-300)) /
                        np.maximum(kap, 1e-300))
    dO = np.zeros((R, N_OUT))
    dO[:, :48] = (-(eta_scale / R) * (x - a_over_k * eta)).reshape(R, 48)
    dO = rb(dO)
    d = [None, None, None]
    d[2] = rb((dO @ wb[3]) * (1 - hs[3] ** 2))
    d[1] = rb((d[2] @ wb[2]) * (1 - hs[2] ** 2))
    d[0] = rb((d[1] @ wb[1]) * (1 - hs[1] ** 2))
    m = masks()
    gw = [d[0].T @ hs[0] * m[0], d[1].T @ hs[1] * m[1], d[2].T @ hs[2] * m[2], dO.T @ hs[3] * m[3]]
    gb = [d[0].sum(0), d[1].sum(0), d[2].sum(0), dO.sum(0)]
    return loss, np.concatenate([g.ravel() for g in gw] + gb)


def random_params(seed, scale_out=0.1):
    rng = np.random.default_rng(seed)
    m = masks()
    fan = [N_FEAT, N_HID, N_HID, N_HID]
    ws = [rng.normal(size=m[l].shape) / np.sqrt(fan[l]) * (scale_out if l == 3 else 1.0) * m[l] for l in range(4)]
    bs = [rng.normal(size=(n,)) * 0.05 for n in (N_HID, N_HID, N_HID, N_OUT)]
    return np.concatenate([w.ravel() for w in ws] + bs).astype(np.float32)


def random_windows(R, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(R, 64, 3)) + np.array([0.0, 0.0, 1.5])
    v /= np.linalg.norm(v, axis=-1, keepdims=True)
    return v.reshape(R, 192).astype(np.float32)


def patch_energy_change(lat, emomM, k, x0, y0, new_patch):
    """Exact dE (units T muB, i.e. mRy-scaled couplings times moments) of replacing the
    4 x 4 patch at (x0, y0) of ensemble k by `new_patch` (16, 3) unit vectors, from the
    full energy difference over the bonds and sites it touches."""
    L = int(round(np.sqrt(lat.natom)))
    mm = lat.mmom[0] if lat.mmom.ndim == 2 else lat.mmom
    sites = [((x0 + px) % L) + L * ((y0 + py) % L) for py in range(4) for px in range(4)]
    old = emomM[k].copy()
    new = old.copy()
    for s, i in enumerate(sites):
        new[i] = new_patch[s] * mm[i]

    def local_energy(m):
        E = 0.0
        seen = set()
        for i in sites:
            ih = lat.aham[i] - 1
            for q in range(lat.nlistsize[ih]):
                j = lat.nlist[i, q] - 1
                key = (min(i, j), max(i, j), "x")
                if key in seen:
                    continue
                seen.add(key)
                E -= lat.ncoup[ih, q] * np.dot(m[i], m[j])
            if lat.do_dm:
                for q in range(lat.dmlistsize[ih]):
                    j = lat.dmlist[i, q] - 1
                    key = (min(i, j), max(i, j), "d")
                    if key in seen:
                        continue
                    seen.add(key)
                    E -= np.dot(lat.dm_vect[ih, q], np.cross(m[i], m[j]))
            E -= np.dot(lat.extfield[0, i] if lat.extfield.ndim == 3 else lat.extfield[i], m[i])
        return E

    return local_energy(new) - local_energy(old)
