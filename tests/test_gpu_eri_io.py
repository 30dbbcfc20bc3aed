"""GPU tests of the integral input path: int/ERI.bin and the 8-fold packed int/ERI_chem.bin
(utils/read_2e_integrals.f90) read into device memory, and the AO->MO transform on device
buffers, chained into a G0W0 that is compared with the oracle."""
import numpy as np
import pytest

from oracle import qkgw_oracle as O
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu


def pack_s8(chem):
    """8-fold packing of chemist integrals (pq|rs), 0-based: pair(i,j) = i(i+1)/2 + j (i >= j),
    then the same over the pairs -- the order AOtoMO/Hartree_matrix_AO_basis.f90:71-93 reads."""
    N = chem.shape[0]
    npair = N * (N + 1) // 2
    out = np.empty(npair * (npair + 1) // 2)
    pairs = [(i, j) for i in range(N) for j in range(i + 1)]
    for P, (i, j) in enumerate(pairs):
        for Q in range(P + 1):
            k, l = pairs[Q]
            out[P * (P + 1) // 2 + Q] = chem[i, j, k, l]
    return out


def _chem_and_phys(N, naux, seed):
    s = synth.small_system(N, max(1, N // 8), naux, seed)
    L = s["L"]
    chem = np.einsum("Ppq,Prs->pqrs", L, L)
    phys = chem.transpose(0, 2, 1, 3)        # <pq|rs> = (pr|qs)
    return s, chem, phys


def test_read_eri_bin_and_chem_bin(ctx, tmp_path):
    import torch
    N = 14
    s, chem, phys = _chem_and_phys(N, 30, 51)
    (tmp_path / "int").mkdir()
    np.asfortranarray(phys).ravel(order="F").tofile(tmp_path / "int" / "ERI.bin")
    pack_s8(chem).tofile(tmp_path / "int" / "ERI_chem.bin")
    ref = np.asfortranarray(phys).ravel(order="F")
    d = torch.empty(N ** 4, dtype=torch.float64, device="cuda")
    api.read_eri_bin(tmp_path / "int" / "ERI.bin", N, d.data_ptr(), ctx=ctx)
    assert np.array_equal(d.cpu().numpy(), ref)
    d.zero_()
    api.read_eri_chem_bin(tmp_path / "int" / "ERI_chem.bin", N, d.data_ptr(), ctx=ctx)
    assert np.array_equal(d.cpu().numpy(), ref)
    with pytest.raises(api.QkError) as ei:  # a file one integral short
        pack_s8(chem)[:-1].tofile(tmp_path / "int" / "short.bin")
        api.read_eri_chem_bin(tmp_path / "int" / "short.bin", N, d.data_ptr(), ctx=ctx)
    assert ei.value.code == api.QK_ERR_ARG
    with pytest.raises(api.QkError):
        api.read_eri_bin(tmp_path / "int" / "missing.bin", N, d.data_ptr(), ctx=ctx)


def test_ao_to_mo_on_device_then_g0w0(ctx, tmp_path):
    import torch
    N, nO = 16, 3
    s, chem, phys = _chem_and_phys(N, 32, 52)
    rng = np.random.default_rng(52)
    c, _ = np.linalg.qr(rng.standard_normal((N, N)))   # orthogonal "MO coefficients"
    (tmp_path / "int").mkdir()
    pack_s8(chem).tofile(tmp_path / "int" / "ERI_chem.bin")
    dAO = torch.empty(N ** 4, dtype=torch.float64, device="cuda")
    api.read_eri_chem_bin(tmp_path / "int" / "ERI_chem.bin", N, dAO.data_ptr(), ctx=ctx)
    dc = torch.from_numpy(np.asfortranarray(c).ravel(order="F")).cuda()
    dMO = torch.empty(N ** 4, dtype=torch.float64, device="cuda")
    api.AOtoMO_ERI_RHF_dev(N, N, dc.data_ptr(), dAO.data_ptr(), dMO.data_ptr(), ctx=ctx)
    ref_mo = O.AOtoMO_ERI_RHF(N, N, c, phys)
    got = dMO.cpu().numpy().reshape((N, N, N, N), order="F")
    assert np.max(np.abs(got - ref_mo)) < 1e-12 * max(1.0, np.max(np.abs(ref_mo)))
    assert np.array_equal(dAO.cpu().numpy(), np.asfortranarray(phys).ravel(order="F"))
    nS = nO * (N - nO)
    de = torch.from_numpy(s["eHF"]).cuda()
    out = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(3)]
    dOm = torch.empty(nS, dtype=torch.float64, device="cuda")
    api.RG0W0_dev(api.GWOptions(linearize=True), N, 0, nO, 0, dMO.data_ptr(), de.data_ptr(),
                  out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), dOm.data_ptr(), ctx=ctx)
    ref = O.RG0W0(True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, ref_mo, s["eHF"])
    assert np.max(np.abs(out[0].cpu().numpy() - ref["eGW"])) < 1e-8


def test_eri_chem_bin_into_qsgw(ctx, tmp_path):
    """The AO integrals of an H chain written as QuAcK's packed int/ERI_chem.bin, read straight
    into device memory and handed to the device-pointer qsGW: the same result as the oracle on
    the in-memory integrals."""
    import torch
    sy = synth.hchain_system(4)
    n, nO = sy["nBas"], sy["nO"]
    chem = sy["ERI_AO"].transpose(0, 2, 1, 3)          # (pq|rs) = <pr|qs>
    (tmp_path / "int").mkdir()
    pack_s8(chem).tofile(tmp_path / "int" / "ERI_chem.bin")
    dERI = torch.empty(n ** 4, dtype=torch.float64, device="cuda")
    api.read_eri_chem_bin(tmp_path / "int" / "ERI_chem.bin", n, dERI.data_ptr(), ctx=ctx)

    def dev(a):
        return torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()

    d = {k: dev(sy[k]) for k in ("eHF", "cHF", "PHF", "S", "T", "V", "Hc", "X")}
    eGW = torch.empty(n, dtype=torch.float64, device="cuda")
    c = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P = torch.empty(n * n, dtype=torch.float64, device="cuda")
    Z = torch.empty(n, dtype=torch.float64, device="cuda")
    opts = api.GWOptions(maxSCF=64, thresh=1e-5, max_diis=5, eta=0.05)
    r = api.qsRGW_dev(opts, n, 0, nO, 0, *[d[k].data_ptr() for k in ("eHF", "cHF", "PHF", "S", "T",
                                                                      "V", "Hc", "X")],
                      dERI.data_ptr(), eGW.data_ptr(), c.data_ptr(), P.data_ptr(), Z.data_ptr(),
                      ctx=ctx)
    torch.cuda.synchronize()
    ref = O.qsRGW(64, 1e-5, 5, 0.05, False, n, n, 0, nO, n - nO, 0, nO * (n - nO), sy["eHF"],
                  sy["cHF"], sy["PHF"], sy["S"], sy["T"], sy["V"], sy["Hc"], sy["X"], sy["ERI_AO"])
    assert r["nSCF"] == ref["nSCF"]
    assert np.max(np.abs(eGW.cpu().numpy() - ref["eGW"])) < 1e-8
    assert abs(r["EqsGW"] - ref["EqsGW"]) < 1e-8
