"""Parity of the native batched path (include/fwi.h) on the GPU.

REF_COMPAT against the golden fixtures made from the reference's kernels;
EXACT against the FP64 exact-adjoint oracle.  Tolerances (relative L2):
  - forward traces vs the reference: 1e-5;
  - REF_COMPAT gradient vs the reference's gradient: 1e-4;
  - EXACT FP64 GPU vs FP64 oracle: 1e-10;  EXACT FP32 GPU vs FP64 oracle: 1e-4;
  - FP16 / BF16 image storage vs FP32 storage: 2e-3 / 2e-2 (stated, measured);
  - misfit (FP64 accumulation) vs the reference's FP32 host sum: 1e-5.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_small.npz"))
NX, NZ, NT, CPML, SZ = (int(G[k]) for k in ("nx", "nz", "nt", "cpml", "sz"))
DH, DT, F = float(G["dh"]), float(G["dt"]), float(G["f"])


def rel_l2(a, b):
    return float(np.linalg.norm((np.asarray(a) - b).ravel()) / np.linalg.norm(np.asarray(b).ravel()))


def ref_shots(nt=NT):
    from fwi_gb300 import make_shots
    return make_shots([(int(sx) - 1, SZ - 1, SZ - 1, CPML, NX - CPML, nt) for sx in G["shots_sx"]])


def ref_ctx(**kw):
    from fwi_gb300 import Context, MODE_REF_COMPAT
    args = dict(nx=NX, nz=NZ, dh=DH, dt=DT, cpml=CPML, f_cpml=F, nt_max=NT, max_shots=2,
                mode=MODE_REF_COMPAT)
    args.update(kw)
    ctx = Context(**args)
    ctx.set_wavelet(G["source"])
    return ctx


def obs_ref():
    return np.concatenate([G["obs"][k][:, CPML:NX - CPML].ravel() for k in range(2)])


def test_forward_traces_match_reference():
    ctx = ref_ctx()
    ctx.set_model(G["vh_t"], G["vp_t"], G["vn_t"])
    tr = ctx.forward(ref_shots()).reshape(2, NT, NX - 2 * CPML)
    for k in range(2):
        assert rel_l2(tr[k], G["obs"][k][:, CPML:NX - CPML]) <= 1e-5


def test_forward_from_vti_parameters():
    ctx = ref_ctx()
    ctx.set_model_vti(G["vel_t"], G["eps_t"], G["del_t"])
    vh, vp, vn = ctx.get_model()
    assert rel_l2(vh, G["vh_t"]) < 1e-7 and rel_l2(vp, G["vp_t"]) < 1e-7 and rel_l2(vn, G["vn_t"]) < 1e-7


@pytest.mark.parametrize("batch", [1, 2])
@pytest.mark.parametrize("strip_pass", [False, True])
def test_ref_compat_gradient_matches_reference(batch, strip_pass, monkeypatch):
    """Both layer-tile paths: memory variables advanced in the layer tiles (the
    default where the tile grid allows it) and by the separate strip pass."""
    if strip_pass:
        monkeypatch.setenv("FWI_INLINE_STRIP", "0")
    ctx = ref_ctx(max_shots=batch)
    ctx.set_model(G["vh_i"], G["vp_i"], G["vn_i"])
    J, gh, gp, gn = ctx.gradient(ref_shots(), obs_ref())
    assert abs(J - float(G["fi_total"])) <= 1e-5 * float(G["fi_total"])
    assert rel_l2(gh, G["gcx"]) <= 1e-4
    assert rel_l2(gp, G["gcz"]) <= 1e-4
    assert rel_l2(gn, G["gdx"]) <= 1e-4


@pytest.mark.parametrize("sprec,tol", [(1, 2e-3), (2, 2e-2)])
def test_reduced_precision_image_storage(sprec, tol):
    ctx = ref_ctx()
    ctx.set_model(G["vh_i"], G["vp_i"], G["vn_i"])
    ref = ctx.gradient(ref_shots(), obs_ref())
    ctx2 = ref_ctx(store_prec=sprec)
    ctx2.set_model(G["vh_i"], G["vp_i"], G["vn_i"])
    low = ctx2.gradient(ref_shots(), obs_ref())
    assert low[0] == ref[0]  # the misfit does not touch the images
    for a, b in zip(low[1:], ref[1:]):
        assert rel_l2(a, b) <= tol


F32_DT, F32_R = float(np.float32(1e-3)), float(np.float32(1e-6))


def exact_problem(seed=9, nx=72, nz=56, nt=260, dtype=np.float64):
    rng = np.random.default_rng(seed)
    vel = 1900 + 700 * rng.random((nz, nx))
    for _ in range(4):
        vel = (vel + np.roll(vel, 1, 0) + np.roll(vel, 1, 1)) / 3
    eps = 0.15 + 0.05 * rng.random((nz, nx))
    dl = 0.05 + 0.05 * rng.random((nz, nx))
    vp = vel ** 2
    # dt and R as the FP32 configuration holds them, so that FP64 runs compare exactly
    return dict(nx=nx, nz=nz, nt=nt, cpml=12, dh=10.0, dt=F32_DT, f=20.0,
                vh=(vp * (1 + 2 * eps)).astype(dtype), vp=vp.astype(dtype),
                vn=(vp * (1 + 2 * dl)).astype(dtype))


def exact_shots(p):
    nx, nz = p["nx"], p["nz"]
    # two windows of different width and length, receivers inside the layers too
    return [dict(sx=20, sz=6, rz=6, rx0=4, rx1=nx - 4, nt=p["nt"], x0=0, nxw=0),
            dict(sx=44, sz=nz - 8, rz=5, rx0=30, rx1=nx - 6, nt=p["nt"] - 40, x0=14, nxw=nx - 16)]


def oracle_exact(p, shots, obs, mask):
    """FP64 oracle on each shot's window, gradients placed back on the model grid."""
    J = 0.0
    g = [np.zeros((p["nz"], p["nx"])) for _ in range(3)]
    o = m = 0
    for s in shots:
        x0 = s["x0"]
        w = s["nxw"] or p["nx"]
        nrec = s["rx1"] - s["rx0"]
        ax, bx, az, bz = po.cpml_profiles(w, p["nz"], p["cpml"], p["dh"], p["dt"], p["f"], R=F32_R,
                                          dtype=np.float64)
        prob = dict(nx=w, nz=p["nz"], nt=s["nt"], cpml=p["cpml"], dh=p["dh"], dt=p["dt"], ax=ax, bx=bx,
                    az=az, bz=bz, source=wavelet(p)[:s["nt"]],
                    vh=np.ascontiguousarray(p["vh"][:, x0:x0 + w], np.float64),
                    vp=np.ascontiguousarray(p["vp"][:, x0:x0 + w], np.float64),
                    vn=np.ascontiguousarray(p["vn"][:, x0:x0 + w], np.float64))
        ob = obs[o:o + s["nt"] * nrec].reshape(s["nt"], nrec)
        Js, gh, gp, gn = po.exact_gradient(prob, s["sx"] - x0, s["sz"], s["rz"], s["rx0"] - x0, s["rx1"] - x0,
                                           obs=ob, mask=mask[m:m + nrec])
        J += Js
        for a, b in zip(g, (gh, gp, gn)):
            a[:, x0:x0 + w] += b
        o += s["nt"] * nrec
        m += nrec
    return J, g


def wavelet(p):
    return po.ricker(p["nt"], p["dt"], p["f"], dtype=np.float64)


def run_exact(p, shots, obs, mask, precision, batch=2, sprec=0):
    from fwi_gb300 import Context, MODE_EXACT, make_shots
    ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"],
                  nt_max=p["nt"], max_shots=batch, mode=MODE_EXACT, precision=precision, store_prec=sprec)
    dt_ = ctx.dtype
    ctx.set_wavelet(wavelet(p).astype(dt_))
    ctx.set_model(*(np.ascontiguousarray(p[k], dt_) for k in ("vh", "vp", "vn")))
    return ctx, ctx.gradient(make_shots(shots), np.ascontiguousarray(obs, dt_), mask)


@pytest.fixture(scope="module")
def exact_case():
    p = exact_problem()
    shots = exact_shots(p)
    true = dict(p, vh=p["vh"] * 1.03, vp=p["vp"] * 0.98, vn=p["vn"] * 1.02)
    from fwi_gb300 import Context, MODE_EXACT, PREC_FP64, make_shots
    ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"],
                  nt_max=p["nt"], max_shots=2, mode=MODE_EXACT, precision=PREC_FP64)
    ctx.set_wavelet(wavelet(p))
    ctx.set_model(true["vh"], true["vp"], true["vn"])
    obs = ctx.forward(make_shots(shots))
    mask = np.ones(sum(s["rx1"] - s["rx0"] for s in shots), np.uint8)
    mask[::9] = 0
    J, g = oracle_exact(p, shots, obs, mask)
    return p, shots, obs, mask, J, g


def test_exact_fp64_matches_fp64_oracle(exact_case):
    from fwi_gb300 import PREC_FP64
    p, shots, obs, mask, J, g = exact_case
    _, (Jg, *gg) = run_exact(p, shots, obs, mask, PREC_FP64)
    assert abs(Jg - J) <= 1e-10 * J
    for a, b in zip(gg, g):
        assert rel_l2(a, b) <= 1e-10


@pytest.mark.parametrize("batch,strip_pass", [(2, False), (1, False), (1, True)])
def test_exact_fp32_within_1e4_of_fp64_oracle(exact_case, batch, strip_pass, monkeypatch):
    """batch 2 mixes two windows (one tile grid from the origin, strip pass);
    batch 1 gives each batch one window (tile grid placed so that the layer
    tiles advance the memory variables), or the strip pass when forced."""
    from fwi_gb300 import PREC_FP32
    if strip_pass:
        monkeypatch.setenv("FWI_INLINE_STRIP", "0")
    p, shots, obs, mask, J, g = exact_case
    _, (Jg, *gg) = run_exact(p, shots, obs, mask, PREC_FP32, batch=batch)
    assert abs(Jg - J) <= 1e-5 * J
    for a, b in zip(gg, g):
        assert rel_l2(a, b) <= 1e-4


def test_exact_batch_size_does_not_change_results(exact_case):
    from fwi_gb300 import PREC_FP32
    p, shots, obs, mask, _, _ = exact_case
    _, one = run_exact(p, shots, obs, mask, PREC_FP32, batch=1)
    _, two = run_exact(p, shots, obs, mask, PREC_FP32, batch=2)
    _, again = run_exact(p, shots, obs, mask, PREC_FP32, batch=2)
    # batch 1 runs each window on its own tile grid (memory variables advanced in
    # the layer tiles), batch 2 one grid for both windows (strip pass): the same
    # arithmetic up to FP32 rounding, which the 260 steps carry to ~1e-6
    assert abs(one[0] - two[0]) <= 1e-5 * abs(two[0])
    assert again[0] == two[0]
    for a, b, c in zip(one[1:], two[1:], again[1:]):
        assert np.array_equal(b, c)  # deterministic
        assert rel_l2(a, b) <= 1e-5


def test_exact_gradient_finite_differences_fp64(exact_case):
    from fwi_gb300 import PREC_FP64, make_shots
    p, shots, obs, mask, _, _ = exact_case
    ctx, (J0, *g) = run_exact(p, shots, obs, mask, PREC_FP64)
    rng = np.random.default_rng(4)
    scale = float(p["vp"].mean()) * 1e-3
    for _ in range(2):
        dm = [rng.standard_normal(p["vh"].shape) * scale for _ in range(3)]
        pred = sum(float((a * b).sum()) for a, b in zip(g, dm))
        e = 1e-2

        def J(sg):
            ctx.set_model(*(np.ascontiguousarray(p[k] + sg * d) for k, d in zip(("vh", "vp", "vn"), dm)))
            return ctx.misfit(make_shots(shots), obs, mask)
        fd = (J(e) - J(-e)) / (2 * e)
        assert abs(fd / pred - 1) < 1e-4


def test_gradient_vti_chain_rule(exact_case):
    from fwi_gb300 import PREC_FP64
    p, shots, obs, mask, _, _ = exact_case
    ctx, (_, gh, gp, gn) = run_exact(p, shots, obs, mask, PREC_FP64)
    gv, ge, gd = ctx.gradient_vti()
    vel = np.sqrt(p["vp"])
    ope, opd = p["vh"] / p["vp"], p["vn"] / p["vp"]
    np.testing.assert_allclose(gv, 2 * vel * (gp + ope * gh + opd * gn), rtol=1e-10, atol=1e-300)
    np.testing.assert_allclose(ge, 2 * p["vp"] * gh, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(gd, 2 * p["vp"] * gn, rtol=1e-12, atol=1e-300)


def test_misfit_only_equals_gradient_misfit(exact_case):
    from fwi_gb300 import PREC_FP32, make_shots
    p, shots, obs, mask, _, _ = exact_case
    ctx, (J, *_g) = run_exact(p, shots, obs, mask, PREC_FP32)
    assert ctx.misfit(make_shots(shots), obs.astype(np.float32), mask) == J


def test_lbfgs_matches_reference_two_loop():
    """fwi_first_step / fwi_lbfgs_direction / fwi_lbfgs_update on the fixtures'
    gradients against src/main.c's iteration 0 and 1 (FP64 dots here, FP32 there)."""
    ctx = ref_ctx()
    ctx.set_model(G["vh_i"], G["vp_i"], G["vn_i"])
    ctx.set_gradient(G["gcx"], G["gcz"], G["gdx"])
    ctx.first_step(3e5, 2e5, 2.5e5)
    vh1, vp1, vn1 = ctx.get_model()
    for a, k in ((vh1, "vh_1"), (vp1, "vp_1"), (vn1, "vn_1")):
        assert rel_l2(a - G[k.replace("_1", "_i")], G[k] - G[k.replace("_1", "_i")]) <= 1e-5
    ctx.set_model(G["vh_1"], G["vp_1"], G["vn_1"])
    ctx.set_gradient(G["gcx_1"], G["gcz_1"], G["gdx_1"])
    st = ctx.lbfgs_direction(5)
    np.testing.assert_allclose(st[0:3], G["lb0_gamma"][[2, 0, 1]], rtol=1e-4)
    ctx.lbfgs_update(1.0, 1.0, 1.0)
    vh2, vp2, vn2 = ctx.get_model()
    for a, k in ((vp2, "vp"), (vn2, "vn"), (vh2, "vh")):
        assert rel_l2(a[16:] - G[f"{k}_1"][16:], G[f"{k}_2"][16:] - G[f"{k}_1"][16:]) <= 1e-4
    ctx.restore_model()
    assert np.array_equal(ctx.get_model()[1], G["vp_1"])


def test_errors_are_reported_not_faulted():
    from fwi_gb300 import FwiError, make_shots
    ctx = ref_ctx()
    with pytest.raises(FwiError) as e:
        ctx.gradient(ref_shots(), obs_ref())  # no model yet
    assert e.value.status == -4
    ctx.set_model(G["vh_i"], G["vp_i"], G["vn_i"])
    bad = make_shots([(0, SZ - 1, SZ - 1, CPML, NX - CPML, NT)])  # source in the frame
    with pytest.raises(FwiError) as e:
        ctx.forward(bad)
    assert e.value.status == -1
    too_long = make_shots([(20, SZ - 1, SZ - 1, CPML, NX - CPML, NT + 1)])
    with pytest.raises(FwiError):
        ctx.forward(too_long)


@pytest.mark.parametrize("mode", ["exact", "ref"])
@pytest.mark.parametrize("every,sprec", [(1, 0), (37, 0), (64, 1), (0, 2), (260, 0)])
@pytest.mark.parametrize("batch", [2, 1])
@pytest.mark.usefixtures("tile_path")
def test_checkpointing_reproduces_full_storage_bitwise(exact_case, mode, every, sprec, batch):
    """Segments recomputed from checkpoints give the images a full store keeps,
    so the gradient is bit-identical (uneven nt and windows included; batch 1
    runs the layer tiles that advance the memory variables themselves)."""
    from fwi_gb300 import Context, MODE_EXACT, MODE_REF_COMPAT, PREC_FP32, STORE_CHECKPOINT, STORE_FULL, make_shots
    p, shots, obs, mask, _, _ = exact_case
    res = []
    for store in (STORE_FULL, STORE_CHECKPOINT):
        ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"],
                      nt_max=p["nt"], max_shots=batch, mode=MODE_EXACT if mode == "exact" else MODE_REF_COMPAT,
                      precision=PREC_FP32, store=store, store_prec=sprec, ckpt_every=every)
        ctx.set_wavelet(wavelet(p).astype(np.float32))
        ctx.set_model(*(np.ascontiguousarray(p[k], np.float32) for k in ("vh", "vp", "vn")))
        res.append(ctx.gradient(make_shots(shots), obs.astype(np.float32), mask))
        del ctx
    assert res[0][0] == res[1][0]
    for a, b in zip(res[0][1:], res[1][1:]):
        assert np.array_equal(a, b), rel_l2(b, a)


def rebuild_region_mask(p, shots):
    """Model points inside every shot's CPML-free region (FWI_STORE_BOUNDARY's R)."""
    m = np.ones((p["nz"], p["nx"]), bool)
    for s in shots:
        w = s["nxw"] or p["nx"]
        r = np.zeros_like(m)
        r[4:p["nz"] - p["cpml"], s["x0"] + p["cpml"]:s["x0"] + w - p["cpml"]] = True
        m &= r
    return m


@pytest.mark.parametrize("precision,sprec,tol", [("fp64", 0, 1e-9), ("fp32", 0, 2e-4), ("fp32", 1, 2e-3)])
@pytest.mark.parametrize("mode", ["exact", "ref"])
@pytest.mark.usefixtures("tile_path")
def test_boundary_storage_rebuilds_the_images(exact_case, precision, sprec, tol, mode):
    """FWI_STORE_BOUNDARY: the misfit is the full store's exactly; inside the
    region every shot rebuilds, the gradient is the full store's up to the
    rounding of the backward rebuild (tolerances measured, stated here);
    outside every shot's region it has only the shots that do rebuild there."""
    from fwi_gb300 import (Context, MODE_EXACT, MODE_REF_COMPAT, PREC_FP32, PREC_FP64, STORE_BOUNDARY, STORE_FULL,
                           make_shots)
    p, shots, obs, mask, _, _ = exact_case
    prec = PREC_FP64 if precision == "fp64" else PREC_FP32
    dt_ = np.float64 if precision == "fp64" else np.float32
    res = []
    for store in (STORE_FULL, STORE_BOUNDARY):
        ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"],
                      nt_max=p["nt"], max_shots=2, mode=MODE_EXACT if mode == "exact" else MODE_REF_COMPAT,
                      precision=prec, store=store, store_prec=sprec)
        ctx.set_wavelet(wavelet(p).astype(dt_))
        ctx.set_model(*(np.ascontiguousarray(p[k], dt_) for k in ("vh", "vp", "vn")))
        res.append(ctx.gradient(make_shots(shots), obs.astype(dt_), mask))
        del ctx
    assert res[0][0] == res[1][0]
    inside = rebuild_region_mask(p, shots)
    for a, b in zip(res[0][1:], res[1][1:]):
        assert rel_l2(b[inside], a[inside]) <= tol, rel_l2(b[inside], a[inside])
        assert np.all(np.isfinite(b))


@pytest.mark.parametrize("store", ["full", "checkpoint", "boundary"])
@pytest.mark.parametrize("batch", [2, 1])
@pytest.mark.usefixtures("tile_path")
def test_graph_replay_matches_direct_issue_bitwise(exact_case, store, batch):
    """Batch sections replayed as CUDA graphs (captured on the second call with
    the same launch parameters) give the results of direct issue bit for bit,
    with the same launch count and tile-timing samples; batch 1 keys each
    shot's window and step count separately."""
    from fwi_gb300 import (Context, MODE_EXACT, PREC_FP32, STORE_BOUNDARY, STORE_CHECKPOINT, STORE_FULL,
                           make_shots)
    p, shots, obs, mask, _, _ = exact_case
    st = dict(full=STORE_FULL, checkpoint=STORE_CHECKPOINT, boundary=STORE_BOUNDARY)[store]
    ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"],
                  nt_max=p["nt"], max_shots=batch, mode=MODE_EXACT, precision=PREC_FP32, store=st, store_prec=1,
                  ckpt_every=37 if store == "checkpoint" else 0)
    ctx.set_wavelet(wavelet(p).astype(np.float32))
    ctx.set_model(*(np.ascontiguousarray(p[k], np.float32) for k in ("vh", "vp", "vn")))
    ctx.set_tile_timing(True)
    sh, ob = make_shots(shots), obs.astype(np.float32)
    runs, launches, tiles, recs = [], [], [], []
    for i in range(4):  # direct, captured, replayed, replayed
        try:
            runs.append(ctx.gradient(sh, ob, mask))
        except Exception as e:
            raise AssertionError(f"call {i}: {e}, cudaError {ctx.last_cuda_error()}") from e
        launches.append(ctx.last_launches())
        tiles.append(ctx.last_tile_timing())
        recs.append(ctx.last_recompute_timing())
    replays = ctx.graph_replays()
    traces = [ctx.forward(sh) for _ in range(3)]
    assert ctx.graph_replays() > replays
    ctx.set_graphs(False)
    direct = ctx.gradient(sh, ob, mask)
    direct_launches = ctx.last_launches()
    direct_traces = ctx.forward(sh)
    assert replays == 2 * 2 * (2 // batch)  # two replayed calls x two sections x batches
    assert ctx.graph_stats()[1] == 3 * (2 // batch)  # gradient (2) and forward-only (1) sections
    assert len(set(launches)) == 1 and direct_launches == launches[0]
    for t in tiles[1:]:
        assert np.all(t[[1, 3]] == tiles[0][[1, 3]]) and np.all(t[[0, 2]] > 0)
    # the segment recompute's forward steps: counted and sampled alike in every call (the sampled
    # launches' interior points may be zero: this small grid has no interior tile under the origin a
    # batch of two windows takes)
    for r in recs:
        if store == "checkpoint":
            assert r[2] == recs[0][2] > 0 and r[1] == recs[0][1] and r[0] >= 0
        else:
            assert np.all(r == 0)
    if store == "checkpoint" and batch == 1:
        assert recs[0][1] > 0 and all(r[0] > 0 for r in recs)
    for r in runs:
        assert r[0] == direct[0]
        for a, b in zip(r[1:], direct[1:]):
            assert np.array_equal(a, b)
    for t in traces:
        assert np.array_equal(t, direct_traces)


def edge_cases():
    p = exact_problem(seed=13, nx=64, nz=52, nt=120)
    nx, nz, nt = p["nx"], p["nz"], p["nt"]
    return p, {
        "single receiver": [dict(sx=30, sz=10, rz=12, rx0=40, rx1=41, nt=nt, x0=0, nxw=0)],
        "first interior row and column": [dict(sx=4, sz=4, rz=4, rx0=4, rx1=9, nt=nt, x0=0, nxw=0)],
        "last interior column, deep source": [dict(sx=nx - 5, sz=nz - 5, rz=nz - 5, rx0=nx - 9, rx1=nx - 4, nt=nt,
                                                  x0=0, nxw=0)],
        "window flush with the right edge": [dict(sx=nx - 12, sz=6, rz=5, rx0=nx - 36, rx1=nx - 4, nt=nt,
                                                  x0=nx - 40, nxw=40)],
        "record shorter than the timing sampler": [dict(sx=20, sz=6, rz=5, rx0=4, rx1=nx - 4, nt=6, x0=0, nxw=0)],
        "batch larger than the shots, two windows": [
            dict(sx=20, sz=6, rz=5, rx0=4, rx1=nx - 4, nt=nt, x0=0, nxw=0),
            dict(sx=30, sz=8, rz=6, rx0=14, rx1=50, nt=nt - 20, x0=10, nxw=44),
            dict(sx=40, sz=7, rz=6, rx0=14, rx1=50, nt=nt - 50, x0=10, nxw=44)],
    }


@pytest.mark.parametrize("case", list(edge_cases()[1]))
def test_edge_geometries_match_fp64_oracle(case):
    """FP32 tile path against the FP64 exact-adjoint oracle on edge geometries
    (tolerances as above: gradients 1e-4, misfit 1e-5), with random observed
    data so that the residuals are far above the traces' rounding."""
    from fwi_gb300 import PREC_FP32
    p, cases = edge_cases()
    shots = cases[case]
    rng = np.random.default_rng(5)
    nobs = sum(s["nt"] * (s["rx1"] - s["rx0"]) for s in shots)
    obs = 1e-3 * rng.standard_normal(nobs)
    mask = (rng.random(sum(s["rx1"] - s["rx0"] for s in shots)) > 0.1).astype(np.uint8)
    J, g = oracle_exact(p, shots, obs, mask)
    _, (Jg, *gg) = run_exact(p, shots, obs, mask, PREC_FP32, batch=len(shots) + 1)
    assert abs(Jg - J) <= 1e-5 * J
    for a, b in zip(gg, g):
        assert rel_l2(a, b) <= 1e-4, rel_l2(a, b)


@pytest.mark.parametrize("store", ["full", "checkpoint", "boundary"])
@pytest.mark.usefixtures("tile_path")
def test_groups_of_several_windows_are_bitwise_one_shot_per_block(exact_case, store):
    """The interior passes' groups of several windows (MIXED kernels: per-shot
    tile roles, model columns and gradient slots) give the results of one
    shot per block bit for bit, and the FP64 oracle's within 1e-4."""
    from fwi_gb300 import (Context, MODE_EXACT, PREC_FP32, STORE_BOUNDARY, STORE_CHECKPOINT, STORE_FULL,
                           make_shots)
    p, shots, obs, mask, J, g = exact_case
    st = dict(full=STORE_FULL, checkpoint=STORE_CHECKPOINT, boundary=STORE_BOUNDARY)[store]
    sh = make_shots(shots)
    res = []
    for sg in (1, 2):
        ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"],
                      nt_max=p["nt"], max_shots=2, mode=MODE_EXACT, precision=PREC_FP32, store=st,
                      ckpt_every=37 if store == "checkpoint" else 0)
        ctx.set_wavelet(wavelet(p).astype(np.float32))
        ctx.set_model(*(np.ascontiguousarray(p[k], np.float32) for k in ("vh", "vp", "vn")))
        c = dict(shots_per_group=sg, layer_shots_per_group=1, inline_strip=0)
        ctx.set_tuning(sh, dict(forward=c, adjoint=c))
        res.append(ctx.gradient(sh, obs.astype(np.float32), mask))
        del ctx
    assert res[0][0] == res[1][0]
    for a, b in zip(res[0][1:], res[1][1:]):
        assert np.array_equal(a, b)
    if store == "full":
        assert abs(res[1][0] - J) <= 1e-5 * J
        for a, b in zip(res[1][1:], g):
            assert rel_l2(a, b) <= 1e-4


def test_a_wait_that_gives_up_is_reported_and_the_context_stays_usable(exact_case):
    """Failure detection on the device without a fault: a barrier wait that
    nothing completes gives up after a few polls, the host gets FWI_ERR_CUDA
    from the status word, and the context then computes the gradient a fresh
    context computes, bit for bit."""
    from fwi_gb300 import PREC_FP32, make_shots
    p, shots, obs, mask, _, _ = exact_case
    ctx, first = run_exact(p, shots, obs, mask, PREC_FP32)
    assert ctx.check_bounded_wait(64) == -2  # FWI_ERR_CUDA
    assert ctx.check_bounded_wait(0) == -1   # FWI_ERR_ARG
    again = ctx.gradient(make_shots(shots), np.ascontiguousarray(obs, np.float32), mask)
    assert again[0] == first[0]
    for a, b in zip(again[1:], first[1:]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("cluster", ["1", "0"])
def test_shots_of_uneven_length_batch_by_length_in_any_caller_order(cluster, monkeypatch):
    """A call forms its batches longest shot first (a batch runs as many steps as its longest
    shot): the traces come back in the caller's order, bit for bit whatever that order, and the
    misfit and gradients of a permuted call agree to FP32 rounding (the sums run in another order)."""
    from fwi_gb300 import Context, MODE_EXACT, PREC_FP32, make_shots
    monkeypatch.setenv("FWI_CLUSTER", cluster)  # the cluster path (this window fits) and the tile passes
    p = exact_problem(seed=17, nx=72, nz=56, nt=260)
    nx = p["nx"]
    shots = [dict(sx=20 + 8 * k, sz=6, rz=5, rx0=4, rx1=nx - 4, nt=nt, x0=0, nxw=0)
             for k, nt in enumerate((150, 260, 200, 260, 90))]
    rng = np.random.default_rng(8)
    obs = [1e-3 * rng.standard_normal(s["nt"] * (nx - 8)) for s in shots]
    masks = [(rng.random(nx - 8) > 0.1).astype(np.uint8) for _ in shots]

    def call(idx):
        ctx = Context(nx=nx, nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"], nt_max=p["nt"],
                      max_shots=2, mode=MODE_EXACT, precision=PREC_FP32)
        ctx.set_wavelet(wavelet(p).astype(np.float32))
        ctx.set_model(*(np.ascontiguousarray(p[k], np.float32) for k in ("vh", "vp", "vn")))
        sh = make_shots([shots[k] for k in idx])
        r = ctx.gradient(sh, np.concatenate([obs[k] for k in idx]).astype(np.float32),
                         np.concatenate([masks[k] for k in idx]))
        tr = ctx.forward(sh)
        cuts = np.cumsum([0] + [shots[k]["nt"] * (nx - 8) for k in idx])
        return r, {k: tr[cuts[i]:cuts[i + 1]] for i, k in enumerate(idx)}

    (J0, *g0), t0 = call([0, 1, 2, 3, 4])
    (J1, *g1), t1 = call([4, 2, 0, 3, 1])
    for k in t0:
        assert np.array_equal(t0[k], t1[k])
    assert abs(J1 - J0) <= 1e-6 * J0
    for a, b in zip(g0, g1):
        assert rel_l2(a, b) <= 1e-6, rel_l2(a, b)
