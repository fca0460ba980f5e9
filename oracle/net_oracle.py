"""NumPy restatement of the learned coarse-grid preconditioner -- TEST
INFRASTRUCTURE ONLY (imported by tests/ and __graft_entry__.smoke(), never by
the product path).

The preconditioner has no counterpart in the reference (its CG loops,
SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90:478-523 / 664-702 / 739-775,
are unpreconditioned), so this oracle restates the library's own
definition, independently of the CUDA code:

* the U-Net (parameter layout, 3x3x3 convolutions with zero padding per
  sample, ReLU, 2x average pooling, nearest upsampling, 1x1 output) in
  float64, optionally rounding every stored activation and gradient to BF16
  where the GPU stores BF16 (``bf16=True``), so GPU and oracle differ only by
  FP32 summation order;
* its exact backward pass (pinned by central finite differences in the CPU
  tests);
* the preconditioner z = D^-1 r + P e_c around it: 4x4x4 restriction, input
  features, output scaling and the clamped cell-centred trilinear
  prolongation.

Layouts: a coarse grid of ny x nx x nz cells per sample is an array
[nb, nz, nx, ny, C] (voxel v = i + ny*(j + nx*k), channels last); fine
fields are halo-padded (ny+2, nx+2, nz+2) arrays indexed [i, j, k].
"""
from __future__ import annotations

import numpy as np

CI = [16, 16, 32, 32, 48, 112, 80, 64, 48, 16]
CO = [16, 32, 32, 48, 64, 48, 32, 32, 16, 1]
E0, E1, E2, E3, E4, D3, D2, D1, D0, OUT = range(10)
CATW = [48, 64, 80, 112]
UPW = [32, 32, 48, 64]
ENC = [E0, E1, E2, E3]
DEC = [D0, D1, D2, D3]
NFEAT = 16


def layout():
    """Offsets (weights, biases) of each layer in the flat parameter vector."""
    off, boff, o = [], [], 0
    for l in range(10):
        taps = 1 if l == OUT else 27
        off.append(o)
        o += CO[l] * taps * CI[l]
        boff.append(o)
        o += CO[l]
    return off, boff, o


OFF, BOFF, NPARAM = layout()


def bf16(a):
    """Round to BF16 (round to nearest even) through FP32, as the GPU does."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64).reshape(np.shape(a))


def weights(p, l):
    taps = 1 if l == OUT else 27
    w = np.asarray(p[OFF[l]:OFF[l] + CO[l] * taps * CI[l]], dtype=np.float64)
    return w.reshape(CO[l], taps, CI[l]), np.asarray(p[BOFF[l]:BOFF[l] + CO[l]], dtype=np.float64)


def _taps():
    for t in range(27):
        yield t, t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1  # (t, di: y, dj: x, dk: z)


def conv(x, w, b=None, flip=False):
    """3x3x3 convolution of x [nb, nz, nx, ny, ci] with w [co, 27, ci]."""
    nb, nz, nx, ny, _ = x.shape
    xp = np.zeros((nb, nz + 2, nx + 2, ny + 2, x.shape[4]))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    out = np.zeros((nb, nz, nx, ny, w.shape[0]))
    for t, di, dj, dk in _taps():
        if flip:
            di, dj, dk = -di, -dj, -dk
        out += xp[:, 1 + dk:1 + dk + nz, 1 + dj:1 + dj + nx, 1 + di:1 + di + ny] @ w[:, t, :].T
    if b is not None:
        out += b
    return out


def conv_wgrad(x, g):
    """dW[co, t, ci] = sum_v g[v, co] x[v + o_t, ci]."""
    nb, nz, nx, ny, ci = x.shape
    co = g.shape[4]
    xp = np.zeros((nb, nz + 2, nx + 2, ny + 2, ci))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    gf = g.reshape(-1, co)
    dw = np.zeros((co, 27, ci))
    for t, di, dj, dk in _taps():
        xs = xp[:, 1 + dk:1 + dk + nz, 1 + dj:1 + dj + nx, 1 + di:1 + di + ny].reshape(-1, ci)
        dw[:, t, :] = gf.T @ xs
    return dw


def pool(x):
    nb, nz, nx, ny, c = x.shape
    return x.reshape(nb, nz // 2, 2, nx // 2, 2, ny // 2, 2, c).mean(axis=(2, 4, 6))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def up_bwd(g):
    nb, nz, nx, ny, c = g.shape
    return g.reshape(nb, nz // 2, 2, nx // 2, 2, ny // 2, 2, c).sum(axis=(2, 4, 6))


def level_valid(valid):
    """Valid extents (y, x, z) per level of a zero-padded grid: each level
    halves the previous one's, rounding up."""
    out = [tuple(valid)]
    for _ in range(4):
        out.append(tuple((v + 1) // 2 for v in out[-1]))
    return out


def mask(a, v):
    """Zero the cells of a [nb, nz, nx, ny, C] array beyond valid extents
    v = (y, x, z) (the padding of a padded grid); None: nothing."""
    if v is None:
        return a
    a = a.copy()
    a[:, v[2]:] = 0.0
    a[:, :, v[1]:] = 0.0
    a[:, :, :, v[0]:] = 0.0
    return a


def forward(p, x, rounding=True, valid=None):
    """U-Net forward on x [nb, nz, nx, ny, 16]; returns (out [nb, nz, nx, ny],
    cache of the stored activations).  valid = (y, x, z) extents of a grid
    zero-padded beyond them: every layer's outputs (and upsampled copies)
    stay zero in the padding."""
    R = bf16 if rounding else (lambda a: a)
    x = R(x)
    w16 = {l: (R(weights(p, l)[0]) if l != OUT else weights(p, l)[0], weights(p, l)[1])
           for l in range(10)}
    lv = level_valid(valid) if valid is not None else [None] * 5
    cat = [None] * 4
    pin = [None] * 5
    dec = [None] * 4
    h = x
    for lev in range(4):
        l = ENC[lev]
        e = mask(R(np.maximum(conv(h, *w16[l]), 0.0)), lv[lev])
        cat[lev] = np.concatenate([np.zeros(e.shape[:4] + (UPW[lev],)), e], axis=4)
        pin[lev + 1] = R(pool(e))
        h = pin[lev + 1]
    a4 = mask(R(np.maximum(conv(pin[4], *w16[E4]), 0.0)), lv[4])
    below = a4
    for lev in (3, 2, 1, 0):
        cat[lev][..., :UPW[lev]] = mask(up(below), lv[lev])
        l = DEC[lev]
        dec[lev] = mask(R(np.maximum(conv(cat[lev], *w16[l]), 0.0)), lv[lev])
        below = dec[lev]
    wo, bo = w16[OUT]
    out = dec[0] @ wo[0, 0, :] + bo[0]
    cache = dict(x=x, cat=cat, pin=pin, dec=dec, a4=a4, w=w16)
    return out, cache


def loss_grad(p, x, target, rounding=True):
    """mean (out - target)^2 and its gradient (flat, parameter order)."""
    R = bf16 if rounding else (lambda a: a)
    out, c = forward(p, x, rounding)
    V = out.size
    diff = out - target
    loss = float((diff ** 2).sum() / V)
    grad = np.zeros(NPARAM)
    w = c["w"]

    def put(l, dw, db):
        n = dw.size
        grad[OFF[l]:OFF[l] + n] = dw.ravel()
        grad[BOFF[l]:BOFF[l] + db.size] = db

    dout = 2.0 * diff / V
    d0 = c["dec"][0]
    put(OUT, (dout[..., None] * d0).reshape(-1, 16).sum(axis=0), np.array([dout.sum()]))
    g = R(dout[..., None] * w[OUT][0][0, 0, :] * (d0 > 0))  # pre-activation gradient of D0
    gcat = [None] * 4
    for lev in range(4):
        l = DEC[lev]
        put(l, conv_wgrad(c["cat"][lev], g), g.reshape(-1, CO[l]).sum(axis=0))
        gcat[lev] = conv(g, np.transpose(w[l][0], (2, 1, 0)), flip=True)
        act = c["a4"] if lev == 3 else c["dec"][lev + 1]
        g = R(up_bwd(gcat[lev][..., :UPW[lev]]) * (act > 0))
    put(E4, conv_wgrad(c["pin"][4], g), g.reshape(-1, CO[E4]).sum(axis=0))
    gp = conv(g, np.transpose(w[E4][0], (2, 1, 0)), flip=True)
    for lev in (3, 2, 1, 0):
        l = ENC[lev]
        act = c["cat"][lev][..., UPW[lev]:]
        ge = R((gcat[lev][..., UPW[lev]:] + up(gp) / 8.0) * (act > 0))
        xin = c["x"] if lev == 0 else c["pin"][lev]
        put(l, conv_wgrad(xin, ge), ge.reshape(-1, CO[l]).sum(axis=0))
        if lev > 0:
            gp = conv(ge, np.transpose(w[l][0], (2, 1, 0)), flip=True)
    return loss, grad


# ------------------------------------------------------------ preconditioner

def restrict(a):
    """Means over 4x4x4 blocks of an interior array [i, j, k] -> [ic, jc, kc]."""
    ny, nx, nz = a.shape
    return a.reshape(ny // 4, 4, nx // 4, 4, nz // 4, 4).mean(axis=(1, 3, 5))


def to_cl(a):
    """[i, j, k] (y, x, z) -> channels-last sample [1, nz, nx, ny]."""
    return np.transpose(a, (2, 1, 0))[None]


def from_cl(a):
    return np.transpose(a[0], (2, 1, 0))


def features(r_int, coef_int, bcx0, bcx1, diag_int=None, scale=1.0, pad=16):
    """Input channels [nb=1, nz, nx, ny, 16], s, c_ref and the valid coarse
    extents (y, x, z) from the interior residual and coefficient (fine
    interior arrays [i, j, k]); the coarse grid is zero-padded to multiples
    of `pad`.  With the CnE form's diagonal, channel 5 = x / (1 + x), x =
    R diag / (scale c_ref)."""
    rc = restrict(r_int)
    cc = restrict(coef_int)
    s = float(np.sqrt((rc ** 2).mean()))
    cref = float(cc.mean())
    nyc, nxc, nzc = rc.shape
    f = np.zeros((nyc, nxc, nzc, NFEAT))
    f[..., 0] = rc / s if s > 0 else 0.0
    f[..., 1] = cc / cref
    f[..., 2] = 1.0
    if bcx0 == 1:
        f[:, 0, :, 3] = 1.0
    if bcx1 == 1:
        f[:, -1, :, 4] = 1.0
    if diag_int is not None:
        x = restrict(diag_int) / (scale * cref)
        f[..., 5] = x / (1.0 + x)
    up16 = lambda n: -(-n // pad) * pad
    fp = np.zeros((up16(nyc), up16(nxc), up16(nzc), NFEAT))
    fp[:nyc, :nxc, :nzc] = f
    return np.transpose(fp, (2, 1, 0, 3))[None], s, cref, (nyc, nxc, nzc)


def _interp_axis(n_fine):
    """(lo, hi, w_lo) per fine cell of the clamped cell-centred linear
    interpolation from n_fine / 4 coarse cells."""
    n = n_fine // 4
    fi = np.arange(n_fine)
    pos = (fi + 0.5) / 4.0 - 0.5
    lo = np.floor(pos).astype(int)
    t = pos - lo
    return np.clip(lo, 0, n - 1), np.clip(lo + 1, 0, n - 1), 1.0 - t


def prolong(ec):
    """Trilinear interpolation of a coarse array [ic, jc, kc] to the fine
    interior."""
    out = ec
    for ax in range(3):
        lo, hi, wl = _interp_axis(out.shape[ax] * 4)
        a = np.take(out, lo, axis=ax)
        b = np.take(out, hi, axis=ax)
        shp = [1, 1, 1]
        shp[ax] = -1
        out = wl.reshape(shp) * a + (1.0 - wl.reshape(shp)) * b
    return out


def inv_diag(coef_h, scale, bcx0, bcx1, diag_h=None):
    """1 / diagonal of q = scale * S(p), or of q = diag p - scale * S(p) when
    diag_h is given (halo-padded coefficient K, hk = K/2, face coefficient
    hk_nb + hk_c; y and z faces Neumann, an x face adds its term when it is
    Dirichlet)."""
    hk = 0.5 * np.asarray(coef_h, dtype=np.float64)
    ny, nx, nz = (n - 2 for n in hk.shape)
    I = slice(1, -1)
    kc = hk[I, I, I]
    s = np.zeros_like(kc)
    s[1:] += hk[1:ny, I, I] + kc[1:]
    s[:-1] += hk[2:ny + 1, I, I] + kc[:-1]
    jm = hk[I, 0:nx, I] + kc
    jp = hk[I, 2:nx + 2, I] + kc
    s[:, 1:] += jm[:, 1:]
    s[:, :-1] += jp[:, :-1]
    if bcx0:
        s[:, 0] += jm[:, 0]
    if bcx1:
        s[:, -1] += jp[:, -1]
    s[:, :, 1:] += hk[I, I, 1:nz] + kc[:, :, 1:]
    s[:, :, :-1] += hk[I, I, 2:nz + 1] + kc[:, :, :-1]
    d = -scale * s
    if diag_h is not None:
        d = np.asarray(diag_h, dtype=np.float64)[I, I, I] + scale * s
    return np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 0.0)


def apply_dir(coef_h, p_int, scale, bcx0, bcx1):
    """scale * S(p) on the interior with the search-direction ghost rules
    (y and z faces copy the edge cell, an x face is 0 when Dirichlet, else a
    copy); faces hk_nb + hk_c, hk = K/2, in the order y+, y-, x+, x-, z+, z-."""
    hk = 0.5 * np.asarray(coef_h, dtype=np.float64)
    p = np.pad(np.asarray(p_int, dtype=np.float64), 1, mode="edge")
    if bcx0:
        p[:, 0, :] = 0.0
    if bcx1:
        p[:, -1, :] = 0.0
    I = slice(1, -1)
    kc, pc = hk[I, I, I], p[I, I, I]
    s = (hk[2:, I, I] + kc) * (p[2:, I, I] - pc)
    s = s - (kc + hk[:-2, I, I]) * (pc - p[:-2, I, I])
    s = s + (hk[I, 2:, I] + kc) * (p[I, 2:, I] - pc)
    s = s - (kc + hk[I, :-2, I]) * (pc - p[I, :-2, I])
    s = s + (hk[I, I, 2:] + kc) * (p[I, I, 2:] - pc)
    s = s - (kc + hk[I, I, :-2]) * (pc - p[I, I, :-2])
    return scale * s


OMEGA = 2.3  # weight of the Jacobi step of the multiplicative form (the GPU's)


def pc_apply(p, kout, coef_h, r_h, scale=1.0, bcx0=1, bcx1=1, rounding=True,
             multiplicative=True, omega=OMEGA, diag_h=None):
    """The learned preconditioner on the interior (halo-padded in and out):
    z1 = P e_c, then z = z1 + omega D^-1 (r - A z1) (multiplicative, the
    default) or z = D^-1 r + z1 (additive).  A = scale S (the potential
    form) or, with diag_h, A = diag - scale S (the CnE form: mass channel
    fed, e_c's sign flipped).  Coarse grids are zero-padded to multiples of
    16 for the network."""
    r = r_h[1:-1, 1:-1, 1:-1]
    coef = coef_h[1:-1, 1:-1, 1:-1]
    dg = None if diag_h is None else np.asarray(diag_h, dtype=np.float64)[1:-1, 1:-1, 1:-1]
    f, s, cref, v = features(r, coef, bcx0, bcx1, dg, scale)
    out, _ = forward(p, f, rounding, valid=v)
    sgn = -1.0 if dg is not None else 1.0
    ec = from_cl(out)[:v[0], :v[1], :v[2]] * (sgn * s * kout / (scale * cref))
    z1 = prolong(ec)
    invd = inv_diag(coef_h, scale, bcx0, bcx1, diag_h)
    z = np.zeros_like(r_h)
    if multiplicative:
        az1 = apply_dir(coef_h, z1, scale, bcx0, bcx1)
        if dg is not None:
            az1 = dg * z1 - az1
        z[1:-1, 1:-1, 1:-1] = z1 + omega * (invd * (r - az1))
    else:
        z[1:-1, 1:-1, 1:-1] = invd * r + z1
    return z
