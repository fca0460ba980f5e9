"""Learned coarse-grid preconditioner: training data, training recipe and the
stored weights (no counterpart in the reference, whose CG loops are
unpreconditioned).

The network (``sbm.Net``, kernels in csrc/sbm_net.cu) maps the features of a
residual r on the 4x-coarsened grid to the restricted error R(A^-1 r),
normalised:

    input  f = [R r / s, R K / c_ref, 1, x0 Dirichlet face, x1 Dirichlet face, 0...]
    target t = R(A^-1 r) * scale * c_ref / (s * k_out)

with s = RMS(R r), c_ref = mean(R K) and one constant k_out (stored with
the weights) that brings the targets to unit RMS.  Pairs (r, A^-1 r) come
from the library's own mixed-precision solver on seeded synthetic
microstructures (``synth.microstructure``) and right-hand sides of several
spectra; training runs on the GPU (``Net.train``).

``python -m elsim_gb300.learned --seed 3 --out FILE`` reruns the recipe of
the stored weights ``elsim_gb300/weights/pc_unet.bin`` (recorded in
pc_unet.json: 64^3 and 128^3 stages, seed 3, the best validation score of
the seeds tried; the reductions of the training kernels use atomics, so a
rerun gives weights of similar quality, not the same bits).  A 256^3 stage
was dropped: every new stage starts with a loss spike (its targets are
larger than the first stage's normalisation) and on the held-out solves the
256^3 stage made the network worse.
"""
from __future__ import annotations

import argparse
import time
from pathlib import Path

import numpy as np

from . import sbm, synth

WEIGHTS = Path(__file__).resolve().parent / "weights" / "pc_unet.bin"
MAGIC = b"SBMNET01"   # trained on the potential form only
MAGIC2 = b"SBMNET02"  # also trained on the CnE form: reads input channel 5 (mass)
NFEAT = 16


# ------------------------------------------------------------- features

def restrict(a: np.ndarray) -> np.ndarray:
    """Means over 4x4x4 blocks of an interior array [i, j, k]."""
    ny, nx, nz = a.shape
    return a.reshape(ny // 4, 4, nx // 4, 4, nz // 4, 4).mean(axis=(1, 3, 5))


def features(r_int: np.ndarray, coef_int: np.ndarray, bcx0: int, bcx1: int,
             diag_int: np.ndarray | None = None, scale: float = 1.0):
    """(input [V][16] channels-last float32, s, c_ref) of one residual; with
    the CnE form's diagonal, channel 5 = x / (1 + x), x = R diag / (scale
    c_ref) (the weight of the mass term against the diffusion)."""
    rc = restrict(r_int)
    cc = restrict(coef_int)
    s = float(np.sqrt((rc ** 2).mean()))
    cref = float(cc.mean())
    f = np.zeros(rc.shape + (NFEAT,), dtype=np.float32)
    f[..., 0] = rc / s if s > 0 else 0.0
    f[..., 1] = cc / cref
    f[..., 2] = 1.0
    if bcx0 == sbm.BC_ZERO:
        f[:, 0, :, 3] = 1.0
    if bcx1 == sbm.BC_ZERO:
        f[:, -1, :, 4] = 1.0
    if diag_int is not None:
        x = restrict(diag_int) / (scale * cref)
        f[..., 5] = x / (1.0 + x)
    # [i, j, k, c] -> voxel v = i + ny*(j + nx*k)
    return np.ascontiguousarray(np.transpose(f, (2, 1, 0, 3)).reshape(-1, NFEAT)), s, cref


def target(e_int: np.ndarray, s: float, cref: float, scale: float, kout: float) -> np.ndarray:
    t = restrict(e_int) * (scale * cref / (s * kout))
    return np.ascontiguousarray(np.transpose(t, (2, 1, 0)).reshape(-1).astype(np.float32))


# ------------------------------------------------------------- data

def _smooth(a: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian blur (reflecting edges) of an interior field."""
    if sigma <= 0:
        return a
    r = int(np.ceil(3 * sigma))
    x = np.arange(-r, r + 1)
    w = np.exp(-0.5 * (x / sigma) ** 2)
    w /= w.sum()
    out = a
    for ax in range(3):
        pad = [(0, 0)] * 3
        pad[ax] = (r, r)
        p = np.pad(out, pad, mode="reflect")
        acc = np.zeros_like(out)
        for q, wq in enumerate(w):
            sl = [slice(None)] * 3
            sl[ax] = slice(q, q + out.shape[ax])
            acc += wq * p[tuple(sl)]
        out = acc
    return out


def rhs_family(shape, rng, coef_h, scale=1.0):
    """Right-hand sides of several spectra for one microstructure: white
    noise, Gaussian-smoothed noise (sigma 1..8 cells), a face source like
    the initial residual of the Dirichlet potential solve, and a mixture."""
    ny, nx, nz = shape
    out = []
    out.append(rng.normal(size=shape))
    for sig in (1.0, 2.5, 6.0):
        out.append(_smooth(rng.normal(size=shape), sig))
    face = np.zeros(shape)
    hk = 0.5 * coef_h
    lvl = rng.uniform(0.5, 1.5)
    face[:, -1, :] = -scale * (hk[1:-1, -1, 1:-1] + hk[1:-1, -2, 1:-1]) * lvl
    if rng.uniform() < 0.5:
        face[:, 0, :] = -scale * (hk[1:-1, 0, 1:-1] + hk[1:-1, 1, 1:-1]) * rng.uniform(-1, 1)
    out.append(face)
    out.append(_smooth(rng.normal(size=shape), 3.0) + 0.2 * rng.normal(size=shape))
    return out


def rhs_bv(shape, rng, psi_h, count=10):
    """Right-hand sides like the Butler-Volmer source of the potential
    systems (SBMES:631-641: RHS = -F R AvPx, the reaction rate times the
    interface measure): the interface measure |grad psi| (central
    differences) times a random smooth rate field (Gaussian-smoothed noise,
    sigma 1-6 cells, random offset and sign), `count` of them."""
    g = np.gradient(psi_h, axis=(0, 1, 2))
    avp = np.sqrt(g[0] ** 2 + g[1] ** 2 + g[2] ** 2)[1:-1, 1:-1, 1:-1]
    avp = np.where(avp < 1e-2, 0.0, avp)
    out = []
    for _ in range(count):
        rate = _smooth(rng.normal(size=shape), float(rng.uniform(1.0, 6.0)))
        rate = rate / max(np.abs(rate).max(), 1e-30) + rng.uniform(-0.5, 0.5)
        out.append(avp * rate * rng.choice([-1.0, 1.0]))
    return out


def cne_problem(psi_h: np.ndarray, rng) -> dict:
    """A CnE-form system q = diag p - scale S(p) like the concentration solve
    of either phase (SBMES:515-521): diag = psE = 1 - psi + 1e-6 (electrolyte)
    or psP = psi + 1e-7 (particle), coefficient = diag, scale log-uniform in
    [0.03, 300] (from mass- to diffusion-dominated), Neumann on every face."""
    if rng.uniform() < 0.5:
        diag = 1.0 - psi_h + 1.0e-6
    else:
        diag = psi_h + 1.0e-7
    diag = np.asfortranarray(diag)
    return dict(coef=diag.copy(order="F"), diag=diag, weight=diag.copy(order="F"),
                scale=float(10.0 ** rng.uniform(-1.5, 2.5)))


def make_pairs(n: int, seeds, tol: float = 1e-7, scale: float = 1.0, verbose: bool = False,
               form: int = 0, rhs: str = "family"):
    """(features, s, c_ref, coarse error) for every right-hand side of
    rhs_family on the seeded n^3 microstructures; errors from the library's
    mixed-precision Jacobi-CG.  form 0: the potential operator scale S
    (Dirichlet zero on both x faces); form 1: CnE-form systems (cne_problem,
    Neumann faces, no face source), whose errors enter with the opposite
    sign so that both forms share one convention."""
    feats, errs, meta = [], [], []
    shape = (n, n, n)
    for seed in seeds:
        t0 = time.time()
        rng = np.random.default_rng(1000 + seed)
        frac = float(rng.uniform(0.45, 0.7))
        ms = synth.microstructure(shape, seed=seed, solid_fraction=frac, tunnel=bool(seed % 2))
        if form == 0:
            prob = synth.potential_problem(ms["psi"])
            sc, op, bc, diag = scale, sbm.OP_GENERIC, sbm.BC_ZERO, None
        else:
            prob = cne_problem(ms["psi"], rng)
            sc, op, bc, diag = prob["scale"], sbm.OP_GENERIC_DIAG, sbm.BC_COPY, prob["diag"]
        coef = prob["coef"]
        with sbm.Context(n, n, n) as ctx:
            ctx.upload("coef", coef)
            ctx.upload("weight", prob["weight"])
            if diag is not None:
                ctx.upload("diag", diag)
            if rhs == "bv":
                rhss = rhs_bv(shape, rng, ms["psi"])
            else:
                rhss = rhs_family(shape, rng, coef, sc)
                if form:
                    rhss = rhss[:4] + rhss[5:]  # no Dirichlet face source
            for r in rhss:
                rh = np.zeros(ctx.hshape, order="F")
                rh[1:-1, 1:-1, 1:-1] = r
                ctx.upload("rhs", rh)
                ctx.upload("x", np.zeros(ctx.hshape, order="F"))
                ctx.cg_solve(op=op, bc_x0=bc, bc_x1=bc, scale=sc, tol=tol,
                             stop_rule=sbm.STOP_REL_RES, precision=sbm.PREC_MIXED,
                             precond=sbm.PC_JACOBI)
                e = ctx.download("x")[1:-1, 1:-1, 1:-1]
                f, s, cref = features(r, coef[1:-1, 1:-1, 1:-1], bc, bc,
                                      None if diag is None else diag[1:-1, 1:-1, 1:-1], sc)
                feats.append(f)
                errs.append((-1.0 if form else 1.0) * restrict(e) * (sc * cref / s))
                meta.append((seed, s, cref))
        if verbose:
            print(f"  seed {seed} (form {form}): {time.time() - t0:.1f} s", flush=True)
    return feats, errs, meta


def to_targets(errs, kout: float) -> np.ndarray:
    return np.concatenate([np.transpose(e, (2, 1, 0)).reshape(-1) / kout for e in errs]).astype(
        np.float32)


# ------------------------------------------------------------- weights

def save(path, net: "sbm.Net", info: dict) -> None:
    """Weights file (the format sbm_net_load reads: magic, int64 count,
    float64 k_out, FP32 parameters) and a JSON record of the recipe beside
    it."""
    import json
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    p = net.params().astype("<f4")
    with open(path, "wb") as f:
        f.write(MAGIC2 if getattr(net, "mass", False) else MAGIC)
        f.write(np.int64(p.size).astype("<i8").tobytes())
        f.write(np.float64(net.out_scale).astype("<f8").tobytes())
        f.write(p.tobytes())
    rec = {k: (np.asarray(v).tolist()) for k, v in info.items() if k != "loss"}
    loss = np.asarray(info.get("loss", []), dtype=float)
    if loss.size:
        rec["loss_first_last"] = [float(loss[:20].mean()), float(loss[-20:].mean())]
    path.with_suffix(".json").write_text(json.dumps(rec, indent=1) + "\n")


def read_info(path=None):
    """(parameters, k_out, mass) of a weights file; mass: the network reads
    input channel 5 (trained on the CnE form too)."""
    raw = Path(path or WEIGHTS).read_bytes()
    if raw[:8] not in (MAGIC, MAGIC2):
        raise ValueError("not a weights file of the learned preconditioner")
    n = int(np.frombuffer(raw[8:16], "<i8")[0])
    kout = float(np.frombuffer(raw[16:24], "<f8")[0])
    return np.frombuffer(raw[24:24 + 4 * n], "<f4").copy(), kout, raw[:8] == MAGIC2


def read(path=None):
    """(parameters, k_out) of a weights file."""
    p, kout, _ = read_info(path)
    return p, kout


def load(path=None) -> "sbm.Net":
    """The stored network (default: the weights shipped with the package)."""
    p, kout, mass = read_info(path)
    return sbm.Net(params=p, out_scale=kout, mass=mass)


# ------------------------------------------------------------- training

# Validation structures (edge, seed): used by nothing else (training seeds
# are seed*1000 + n + k, the tests and the benchmark use their own seeds).
VALIDATION = ((128, 900001), (256, 900002))
# CnE-form validation system (edge, seed, scale): diffusion-dominated, the
# electrolyte phase of its structure
VALIDATION_CNE = ((128, 900003, 30.0),)


def cne_validation_problem(n: int, seed: int, scale: float) -> dict:
    """The CnE-form validation system: diag = coefficient = 1 - psi + 1e-6,
    Neumann faces, a smooth right-hand side (seeded)."""
    ms = synth.microstructure((n, n, n), seed=seed, solid_fraction=0.6, tunnel=True)
    diag = np.asfortranarray(1.0 - ms["psi"] + 1.0e-6)
    rng = np.random.default_rng(seed)
    rhs = np.zeros_like(diag, order="F")
    rhs[1:-1, 1:-1, 1:-1] = _smooth(rng.normal(size=(n, n, n)), 3.0)
    return dict(coef=diag.copy(order="F"), diag=diag, weight=diag.copy(order="F"), rhs=rhs,
                x=np.zeros_like(diag, order="F"), scale=scale)


def validation_set(cases=VALIDATION, cne_cases=()):
    """Contexts of the validation solves: potential solves of tunnelled
    structures and, for a network with the mass channel, CnE-form systems."""
    vals = []
    for n, sd in cases:
        ms = synth.microstructure((n, n, n), seed=sd, solid_fraction=0.6, tunnel=True)
        prob = synth.potential_problem(ms["psi"])
        ctx = sbm.Context(n, n, n)
        for k in ("coef", "rhs", "weight"):
            ctx.upload(k, prob[k])
        vals.append((ctx, prob, sbm.OP_GENERIC, sbm.BC_ZERO, 1.0))
    for n, sd, sc in cne_cases:
        prob = cne_validation_problem(n, sd, sc)
        ctx = sbm.Context(n, n, n)
        for k in ("coef", "rhs", "weight", "diag"):
            ctx.upload(k, prob[k])
        vals.append((ctx, prob, sbm.OP_GENERIC_DIAG, sbm.BC_COPY, sc))
    return vals


def validate(net, vals, cap: int = 2000) -> int:
    """Total flexible-CG iterations to rel-res 1e-8 over the validation
    solves with `net` as preconditioner (cap per solve if it fails)."""
    tot = 0
    for ctx, prob, op, bc, sc in vals:
        if getattr(ctx, "_net", None) is not net:
            ctx.set_net(net)
        ctx.upload("x", prob["x"])
        r = ctx.cg_solve(op=op, bc_x0=bc, bc_x1=bc, scale=sc, tol=1e-8, max_it=cap,
                         stop_rule=sbm.STOP_REL_RES, precision=sbm.PREC_MIXED,
                         precond=sbm.PC_LEARNED, raise_on_maxit=False)
        tot += r["iters"] if r["status"] == sbm.OK else cap
    return tot


def train(sizes=((64, 48), (128, 96)), steps=(1500, 12000), batch=(8, 4), lr=(2e-3, 1e-3),
          seed: int = 0, eval_every: int = 500, verbose: bool = True, cne: bool = False,
          rhs: str = "family", cne_only: bool = False):
    """Training recipe of the stored weights: for each (n, structures) stage
    build pairs at n^3 (coarse n/4) and run Adam on the GPU (learning rate
    decayed to 0.3x and 0.1x over the last 40 % and 10 % of the stage); k_out
    from the first stage's targets.  Every `eval_every` steps the network is
    scored by the flexible-CG iterations it needs on the validation solves,
    and the best parameters seen are returned (the MSE of the coarse error is
    only a proxy for the preconditioner's quality).  With cne, every stage
    adds as many CnE-form systems (make_pairs form 1, other seeds) to the
    potential ones, the network reads the mass channel, and a CnE-form
    solve joins the validation score; with cne_only the network sees and is
    scored on CnE-form systems alone.  Returns (net, info)."""
    cne = cne or cne_only
    net = sbm.Net(seed=seed, mass=cne)
    vals = validation_set(cases=() if cne_only else VALIDATION,
                          cne_cases=VALIDATION_CNE if cne else ())
    kout = None
    hist_all, val_hist = [], []
    best, best_p = None, None
    calls = 0
    for (n, nseeds), st, b, eta in zip(sizes, steps, batch, lr):
        t0 = time.time()
        seeds = range(seed * 1000 + n, seed * 1000 + n + nseeds)
        feats, errs = [], []
        if not cne_only:
            feats, errs, _ = make_pairs(n, seeds, verbose=verbose, rhs=rhs)
        if cne:
            f1, e1, _ = make_pairs(n, range(seed * 1000 + 500 + n, seed * 1000 + 500 + n + nseeds),
                                   verbose=verbose, form=1)
            feats += f1
            errs += e1
            del f1, e1
        if kout is None:
            kout = float(np.sqrt(np.mean(np.concatenate([e.ravel() ** 2 for e in errs]))))
            net.out_scale = kout
        net.set_data(np.concatenate(feats), to_targets(errs, kout), (n // 4, n // 4, n // 4))
        del feats, errs
        if verbose:
            print(f"stage n={n}: pairs in {time.time() - t0:.1f} s", flush=True)
        t1 = time.time()
        for part, f in ((0.6, 1.0), (0.3, 0.3), (0.1, 0.1)):
            todo = max(1, int(st * part))
            while todo > 0:
                k = min(eval_every, todo)
                calls += 1
                hist_all.append(net.train_steps(k, b, eta * f, seed=seed * 7919 + calls))
                todo -= k
                v = validate(net, vals)
                val_hist.append(v)
                if best is None or v < best:
                    best, best_p = v, net.params().copy()
        if verbose:
            h = np.concatenate(hist_all)
            print(f"  trained {st} steps in {time.time() - t1:.1f} s; loss {h[:20].mean():.4f}"
                  f" -> {h[-20:].mean():.4f}; validation iterations {val_hist[-1]}"
                  f" (best {best})", flush=True)
    net.set_params(best_p)
    for ctx, *_ in vals:
        ctx.close()
    info = dict(sizes=np.array(sizes), steps=np.array(steps), batch=np.array(batch),
                lr=np.array(lr), seed=seed, eval_every=eval_every, cne=cne, cne_only=cne_only,
                rhs=rhs,
                validation=np.array(VALIDATION),
                validation_cne=np.array(VALIDATION_CNE if cne else []),
                validation_iterations=np.array(val_hist),
                best_validation_iterations=best, loss=np.concatenate(hist_all))
    return net, info


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cne", action="store_true",
                    help="train on CnE-form systems too (the network then reads the mass channel)")
    ap.add_argument("--cne-only", action="store_true",
                    help="train and validate on CnE-form systems alone (mass channel)")
    ap.add_argument("--recipe", default="shipped", choices=["shipped", "bv64"],
                    help="shipped: the recipe of the stored weights (64^3 and 128^3 stages, "
                         "right-hand sides of several spectra); bv64: 2,000 pairs from 200 "
                         "structures of 64^3 with Butler-Volmer-like interface sources")
    a = ap.parse_args(argv)
    if a.recipe == "bv64":
        net, info = train(sizes=((64, 200),), steps=(13500,), batch=(8,), lr=(1.5e-3,),
                          seed=a.seed, cne=a.cne, rhs="bv")
    else:
        net, info = train(seed=a.seed, cne=a.cne, cne_only=a.cne_only)
    save(a.out, net, info)
    print("saved", a.out)


if __name__ == "__main__":
    main()
