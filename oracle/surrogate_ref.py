"""CPU restatement of the learned detector response (test infrastructure).

The GPU path (gpet_gb300/csrc/surrogate.cu) is a new stage with no
counterpart in the reference, which always transports photons through the
panels (gPET_kernals.cu:839-1233). This module is the checker for it: the
same model, loss and backward pass in numpy, either in float64 without
rounding (checked against finite differences) or with the GPU's bf16
rounding points (inputs, weights and activations rounded to bf16; products
accumulated in float, dZ rounded to bf16 before the weight and input
products) for comparison with the tensor-core kernels.

Only tests import it.
"""
import numpy as np

IN, FEAT, HID, OUT, OUT_USED, EMB = 16, 16, 256, 208, 204, 6
EMB_COL = 8             # first input column of the panel embedding
CRY, MIX, BINS = 64, 4, 64
CLASS_BIN = 40          # energy bins >= this take the second crystal set (columns 64-127)
COL_W, COL_MU, COL_LS, COL_E = 128, 132, 136, 140
LAYERS = 5
LS_MIN, LS_MAX = -7.0, 3.0

ENTRY_DTYPE = np.dtype([("panel", "<i4"), ("y", "<f4"), ("z", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"),
                        ("E", "<f4"), ("crystal", "<i4"), ("depth", "<f4"), ("Edep", "<f4")])
assert ENTRY_DTYPE.itemsize == 40


def fan_in(l):
    return IN if l == 0 else HID


def fan_out(l):
    return OUT if l == LAYERS - 1 else HID


def offsets(npanels):
    """(weight offset, bias offset) per layer and the embedding offset."""
    o, lay = 0, []
    for l in range(LAYERS):
        w = o
        o += fan_out(l) * fan_in(l)
        b = o
        o += fan_out(l)
        lay.append((w, b))
    return lay, o, o + npanels * EMB


def unpack(params, npanels):
    lay, emb_off, total = offsets(npanels)
    assert params.size == total
    Ws = [params[w:b].reshape(fan_out(l), fan_in(l)) for l, (w, b) in enumerate(lay)]
    bs = [params[b:b + fan_out(l)] for l, (w, b) in enumerate(lay)]
    emb = params[emb_off:].reshape(npanels, EMB)
    return Ws, bs, emb


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return (((u + r) >> 16) << 16).astype(np.uint32).view(np.float32)


def default_pitch(half_y, half_z, crystal_n):
    """Crystal pitch of a square module of crystal_n crystals without edge gaps."""
    side = int(round(np.sqrt(crystal_n)))
    return 2.0 * half_y / side, 2.0 * half_z / side


def features(rec, emb, half_y, half_z, pitch, depth_len):
    """The 16 inputs: y, z over the half-widths, direction, E / 511 keV, the
    offsets (in pitches, from the crystal centre) of the straight path at half
    the panel depth, the panel embedding, the entry point's offsets (float32
    arithmetic, as on the GPU)."""
    n = len(rec)
    f = np.zeros((n, IN), np.float64)
    y = rec["y"].astype(np.float32)
    z = rec["z"].astype(np.float32)
    f[:, 0] = y / np.float32(half_y)
    f[:, 1] = z / np.float32(half_z)
    f[:, 2] = rec["ux"]
    f[:, 3] = rec["uy"]
    f[:, 4] = rec["uz"]
    f[:, 5] = rec["E"].astype(np.float32) * np.float32(1.0 / 511000.0)
    ux = rec["ux"].astype(np.float32)
    a = np.maximum(np.abs(ux), np.float32(0.05))
    hd = np.float32(0.5) * np.float32(depth_len)
    ym = y + rec["uy"].astype(np.float32) / a * hd
    zm = z + rec["uz"].astype(np.float32) / a * hd
    tym = (ym + np.float32(half_y)) / np.float32(pitch[0])
    tzm = (zm + np.float32(half_z)) / np.float32(pitch[1])
    f[:, 6] = tym - np.floor(tym) - np.float32(0.5)
    f[:, 7] = tzm - np.floor(tzm) - np.float32(0.5)
    f[:, EMB_COL:EMB_COL + EMB] = emb[rec["panel"]]
    ty = (y + np.float32(half_y)) / np.float32(pitch[0])
    tz = (z + np.float32(half_z)) / np.float32(pitch[1])
    f[:, 14] = ty - np.floor(ty) - np.float32(0.5)
    f[:, 15] = tz - np.floor(tz) - np.float32(0.5)
    return f


def targets(rec, depth_len):
    has = (rec["crystal"] >= 0) & (rec["Edep"] > 0)
    cry = np.where(has, rec["crystal"], -1)
    dep = np.where(has, rec["depth"].astype(np.float32) / np.float32(depth_len), 0.0)
    b = np.floor(rec["Edep"].astype(np.float32) / rec["E"].astype(np.float32) * np.float32(BINS)).astype(np.int64)
    b = np.clip(b, 1, BINS - 1)
    return cry, dep.astype(np.float64), np.where(has, b, 0)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _lse(x, axis=-1):
    m = x.max(axis=axis, keepdims=True)
    return (m + np.log(np.exp(x - m).sum(axis=axis, keepdims=True)))


def _xent(out, d, rows, cols, target):
    """Cross entropy of out[rows, cols] against target columns; adds the
    gradient into d and returns the summed loss."""
    c = out[rows[:, None], cols]
    cl = _lse(c)
    loss = (cl[:, 0] - c[np.arange(len(rows)), target]).sum()
    pc = np.exp(c - cl)
    pc[np.arange(len(rows)), target] -= 1.0
    d[rows[:, None], cols] = pc
    return loss


def loss_and_dout(out, cry, dep, b, crystal_n, crystal_ny=None):
    """Mean loss and d loss / d out (float64). A head of more than 64
    crystals is factorised: the first 32 columns of each energy class's set
    are row logits (crystal_ny rows), the last 32 column logits (crystal_n /
    crystal_ny columns), the crystal being row + crystal_ny * column."""
    n = len(out)
    d = np.zeros_like(out)
    e = out[:, COL_E:COL_E + BINS]
    lse = _lse(e)
    loss = (lse[:, 0] - e[np.arange(n), b]).sum()
    pe = np.exp(e - lse)
    pe[np.arange(n), b] -= 1.0
    d[:, COL_E:COL_E + BINS] = pe
    has = cry >= 0
    if has.any():
        i = np.nonzero(has)[0]
        # the crystal set of each sample's energy class
        c0 = np.where(b[i] >= CLASS_BIN, CRY, 0)[:, None]
        if crystal_n > CRY:
            ny = crystal_ny
            nz = crystal_n // ny
            loss += _xent(out, d, i, c0 + np.arange(ny)[None, :], cry[i] % ny)
            loss += _xent(out, d, i, c0 + 32 + np.arange(nz)[None, :], cry[i] // ny)
        else:
            loss += _xent(out, d, i, c0 + np.arange(crystal_n)[None, :], cry[i])
        w = out[i, COL_W:COL_W + MIX]
        lw = w - _lse(w)
        mu = out[i, COL_MU:COL_MU + MIX]
        raw = out[i, COL_LS:COL_LS + MIX]
        ls = np.clip(raw, LS_MIN, LS_MAX)
        x = dep[i][:, None]
        zz = (x - mu) * np.exp(-ls)
        lp = lw - 0.5 * zz * zz - ls - 0.91893853320467274
        plse = _lse(lp)
        loss += (-plse[:, 0]).sum()
        g = np.exp(lp - plse)
        iv = np.exp(-2.0 * ls)
        dx = x - mu
        d[i, COL_W:COL_W + MIX] = np.exp(lw) - g
        d[i, COL_MU:COL_MU + MIX] = -g * dx * iv
        d[i, COL_LS:COL_LS + MIX] = np.where((raw > LS_MIN) & (raw < LS_MAX), -g * (dx * dx * iv - 1.0), 0.0)
    return loss / n, d / n


def forward_backward(params, rec, npanels, half_y, half_z, depth_len, crystal_n, rounding=True, pitch=None,
                     crystal_ny=None):
    """Loss, gradient (flat, like params) and head outputs of the records;
    pitch: the crystal pitch (y, z), default_pitch when None; crystal_ny:
    crystals per row (square grid when None)."""
    p = np.asarray(params, np.float64)
    Ws, bs, emb = unpack(p, npanels)
    r = bf16 if rounding else (lambda x: np.asarray(x, np.float64))
    if pitch is None:
        pitch = default_pitch(half_y, half_z, crystal_n)
    f = features(rec, emb, half_y, half_z, pitch, depth_len)
    x = r(f).astype(np.float64)
    ins, Zs = [x], []
    h = x
    for l in range(LAYERS):
        z = h @ r(Ws[l]).astype(np.float64).T + bs[l]
        if rounding:
            z = z.astype(np.float32).astype(np.float64)
        if l < LAYERS - 1:
            Zs.append(z)
            h = r(silu(z)).astype(np.float64)
            ins.append(h)
        else:
            out = z
    cry, dep, b = targets(rec, depth_len)
    if crystal_ny is None:
        crystal_ny = int(round(np.sqrt(crystal_n)))
    loss, dz = loss_and_dout(out, cry, dep, b, crystal_n, crystal_ny)
    lay, emb_off, total = offsets(npanels)
    g = np.zeros(total, np.float64)
    for l in range(LAYERS - 1, -1, -1):
        dzr = r(dz).astype(np.float64)
        w, bo = lay[l]
        g[w:bo] = (dzr.T @ ins[l]).ravel()
        g[bo:bo + fan_out(l)] = dz.sum(axis=0)
        dinp = dzr @ r(Ws[l]).astype(np.float64)
        if l > 0:
            dz = dinp * silu_grad(Zs[l - 1])
        else:
            ge = np.zeros((npanels, EMB))
            np.add.at(ge, rec["panel"], dinp[:, EMB_COL:EMB_COL + EMB])
            g[emb_off:] = ge.ravel()
    # padding entries carry no gradient
    w0, _ = lay[0]
    g[w0:w0 + fan_out(0) * IN].reshape(fan_out(0), IN)[:, FEAT:] = 0.0
    w4, b4 = lay[LAYERS - 1]
    g[w4:b4].reshape(OUT, HID)[OUT_USED:, :] = 0.0
    g[b4 + OUT_USED:b4 + OUT] = 0.0
    return loss, g, out


def random_records(n, npanels, half_y, half_z, depth_len, crystal_n, seed):
    """Plausible synthetic entry records for gradient checks."""
    rng = np.random.default_rng(seed)
    rec = np.zeros(n, ENTRY_DTYPE)
    rec["panel"] = rng.integers(0, npanels, n)
    rec["y"] = rng.uniform(-half_y, half_y, n)
    rec["z"] = rng.uniform(-half_z, half_z, n)
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    u[:, 0] = -np.abs(u[:, 0])
    rec["ux"], rec["uy"], rec["uz"] = u[:, 0], u[:, 1], u[:, 2]
    rec["E"] = rng.uniform(1.0e5, 5.2e5, n)
    has = rng.uniform(size=n) < 0.8
    rec["crystal"] = np.where(has, rng.integers(0, crystal_n, n), -1)
    rec["depth"] = np.where(has, rng.uniform(0, depth_len, n), 0.0)
    rec["Edep"] = np.where(has, rec["E"] * rng.uniform(0.02, 1.0, n), 0.0)
    return rec


def init_params(npanels, seed):
    rng = np.random.default_rng(seed)
    lay, emb_off, total = offsets(npanels)
    p = np.zeros(total, np.float32)
    for l, (w, b) in enumerate(lay):
        k = FEAT if l == 0 else fan_in(l)
        a = (0.1 if l == LAYERS - 1 else 1.0) / np.sqrt(k)
        W = rng.uniform(-a, a, (fan_out(l), fan_in(l)))
        if l == 0:
            W[:, FEAT:] = 0
        if l == LAYERS - 1:
            W[OUT_USED:, :] = 0
        p[w:b] = W.ravel()
        p[b:b + fan_out(l)] = rng.uniform(-0.05, 0.05, fan_out(l)) * (np.arange(fan_out(l)) < (
            OUT_USED if l == LAYERS - 1 else fan_out(l)))
    p[emb_off:] = rng.uniform(-0.1, 0.1, total - emb_off)
    return p
