"""fwi_residual_misfit_noalloc: the residual + FP64 misfit reduction for callers
that cannot let the library allocate device memory (drivers that allocate
every buffer up front, as the reference's main.c does, or processes whose
device memory belongs to another allocator).  Its scratch is a fixed array in
the library; its results must equal the context path's (fwi_misfit) within
the FP64 summation-order tolerance, call after call.

Collected last (file name) so that a run stopping at the first failure has
already run every other test."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_small.npz"))
NX, NZ, NT, CPML, SZ = (int(G[k]) for k in ("nx", "nz", "nt", "cpml", "sz"))


def call(L, res, syn, obs, mask, nt, nrec, mis):
    return L.fwi_residual_misfit_noalloc(res.data_ptr(), syn.data_ptr(), obs.data_ptr(),
                                         None if mask is None else mask.data_ptr(), nt, nrec, mis.data_ptr(), None)


def test_noalloc_misfit_matches_context_path_twice():
    torch = pytest.importorskip("torch")
    import fwi_gb300
    from fwi_gb300 import native
    L = native.lib()
    ctx = fwi_gb300.Context(nx=NX, nz=NZ, dh=float(G["dh"]), dt=float(G["dt"]), cpml=CPML,
                            f_cpml=float(G["f"]), nt_max=NT, max_shots=2, mode=fwi_gb300.MODE_EXACT)
    ctx.set_wavelet(G["source"])
    ctx.set_model(G["vh_i"], G["vp_i"], G["vn_i"])
    nrec = NX - 2 * CPML
    shots = fwi_gb300.make_shots([(int(sx) - 1, SZ - 1, SZ - 1, CPML, NX - CPML, NT) for sx in G["shots_sx"]])
    obs = np.concatenate([G["obs"][k][:, CPML:NX - CPML].ravel() for k in range(2)]).astype(np.float32)
    mask = np.ones(2 * nrec, np.uint8)
    mask[5::11] = 0
    J_ctx = ctx.misfit(shots, obs, mask)
    J_ctx_nomask = ctx.misfit(shots, obs, None)

    syn = torch.zeros(2 * NT * nrec, dtype=torch.float32, device="cuda")
    ctx.forward(shots, out=syn)
    obs_d = torch.from_numpy(obs).cuda()
    # the two shots share nrec and the same mask pattern per shot here
    assert np.array_equal(mask[:nrec], mask[nrec:])
    mask_d = torch.from_numpy(mask[:nrec].copy()).cuda()
    res = torch.full_like(syn, float("nan"))
    mis = torch.zeros(1, dtype=torch.float64, device="cuda")
    want_res = ((syn - obs_d).view(2 * NT, nrec) * mask_d.to(torch.float32)).view(-1)
    for rep in range(2):
        assert call(L, res, syn, obs_d, mask_d, 2 * NT, nrec, mis) == 0
        torch.cuda.synchronize()
        J = float(mis.item())
        assert abs(J - J_ctx) <= 1e-12 * J_ctx, (rep, J, J_ctx)
        assert torch.equal(res, want_res)
        res.fill_(float("nan"))
        mis.zero_()

    # no mask: every trace counts, against the context path and an FP64 sum here of the
    # FP32 differences (the residual is an FP32 array; its squares accumulate in FP64)
    d64 = (syn - obs_d).double()
    want_nomask = 0.5 * float((d64 * d64).sum())
    assert call(L, res, syn, obs_d, None, 2 * NT, nrec, mis) == 0
    torch.cuda.synchronize()
    J = float(mis.item())
    assert abs(J - J_ctx_nomask) <= 1e-12 * J_ctx_nomask
    assert abs(J - want_nomask) <= 1e-12 * want_nomask
    assert torch.equal(res, syn - obs_d)

    # a request beyond the scratch array's limit is refused before any launch, also when
    # nt * nrec would not fit in a long
    big = call(L, res, syn, obs_d, None, (16384 * 4096) // nrec + 1, nrec, mis)
    assert big == native.FWI_ERR_ARG
    assert call(L, res, syn, obs_d, None, 2 ** 62, nrec, mis) == native.FWI_ERR_ARG


def test_noalloc_partial_blocks_and_changing_sizes_repeat_exactly():
    """Sizes that are not a multiple of one block's 4096 samples and span several
    blocks, alternated, repeat bit for bit: every call starts its completion
    counter from zero, whatever size the call before it had."""
    torch = pytest.importorskip("torch")
    from fwi_gb300 import native
    L = native.lib()
    g = torch.Generator(device="cuda").manual_seed(7)
    for nt, nrec in ((37, 301), (5, 17), (1031, 77), (37, 301), (5, 17), (1031, 77)):
        n = nt * nrec
        syn = torch.randn(n, generator=g, device="cuda")
        obs = torch.randn(n, generator=g, device="cuda")
        res = torch.empty_like(syn)
        mis = torch.zeros(1, dtype=torch.float64, device="cuda")
        assert call(L, res, syn, obs, None, nt, nrec, mis) == 0
        torch.cuda.synchronize()
        d = (syn - obs).double()
        want = 0.5 * float((d * d).sum())
        J = float(mis.item())
        assert abs(J - want) <= 1e-12 * want, (nt, nrec, J, want)
        assert torch.equal(res, syn - obs)
    # the same inputs twice in a row give the same bits
    syn = torch.randn(1031 * 77, generator=g, device="cuda")
    obs = torch.randn(1031 * 77, generator=g, device="cuda")
    res = torch.empty_like(syn)
    mis = torch.zeros(1, dtype=torch.float64, device="cuda")
    got = []
    for _ in range(2):
        assert call(L, res, syn, obs, None, 1031, 77, mis) == 0
        torch.cuda.synchronize()
        got.append(float(mis.item()))
    assert got[0] == got[1]
