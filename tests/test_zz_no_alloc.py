"""fwi_residual_misfit_noalloc: the residual + FP64 misfit reduction for callers
that cannot let the library allocate device memory (drivers that allocate
every buffer up front, as the reference's main.c does, or processes whose
device memory belongs to another allocator).  Its scratch is a fixed array in
the library; its results must equal the context path's (fwi_misfit) within
the FP64 summation-order tolerance, call after call.

Collected last (file name) so that a run stopping at the first failure has
already run every other test."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_small.npz"))
NX, NZ, NT, CPML, SZ = (int(G[k]) for k in ("nx", "nz", "nt", "cpml", "sz"))


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

    syn = torch.zeros(2 * NT * nrec, dtype=torch.float32, device="cuda")
    ctx.forward(shots, out=syn)
    obs_d = torch.from_numpy(obs).cuda()
    # the two shots share nrec and the same mask pattern per shot here
    assert np.array_equal(mask[:nrec], mask[nrec:])
    mask_d = torch.from_numpy(mask[:nrec].copy()).cuda()
    res = torch.full_like(syn, float("nan"))
    mis = torch.zeros(1, dtype=torch.float64, device="cuda")
    want_res = ((syn - obs_d).view(2 * NT, nrec) * mask_d.to(torch.float32)).view(-1)
    for call in range(2):
        rc = L.fwi_residual_misfit_noalloc(res.data_ptr(), syn.data_ptr(), obs_d.data_ptr(),
                                           mask_d.data_ptr(), 2 * NT, nrec, mis.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        J = float(mis.item())
        assert abs(J - J_ctx) <= 1e-12 * J_ctx, (call, J, J_ctx)
        assert torch.equal(res, want_res)
        res.fill_(float("nan"))
        mis.zero_()

    # a request beyond the scratch array's limit is refused before any launch
    big = int(L.fwi_residual_misfit_noalloc(res.data_ptr(), syn.data_ptr(), obs_d.data_ptr(), None,
                                            (16384 * 4096) // nrec + 1, nrec, mis.data_ptr(), None))
    assert big == native.FWI_ERR_ARG
