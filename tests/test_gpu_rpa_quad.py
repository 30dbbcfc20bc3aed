"""GPU tests of the dRPA correlation energy by imaginary-frequency quadrature (the mixed tier's
EcRPA at the G0W0 energies): against the Casida eigenvalues of the oracle (LR/phRLR.f90) on the
same energies, from the factor L and from the ERI tensor (pivoted Cholesky of (ia|jb))."""
import numpy as np
import pytest

from oracle import qkgw_oracle as O
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _ec_oracle(N, nO, e, E):
    nV = N - nO
    nS = nO * nV
    A = O.phRLR_A(1, True, N, 0, nO, nV, 0, nS, 1.0, e, E)
    B = O.phRLR_B(1, True, N, 0, nO, nV, 0, nS, 1.0, E)
    return O.phRLR(False, nS, A, B)[0]


@pytest.mark.parametrize("N,nO,naux,seed", [(48, 6, 48, 31), (80, 10, 60, 32), (64, 8, 192, 33),
                                            (30, 4, 12, 34)])
def test_quadrature_matches_casida_eigenvalues(ctx, N, nO, naux, seed):
    import torch
    s = synth.small_system(N, nO, naux, seed)
    E = synth.eri_phys_numpy(s["L"])
    ref = _ec_oracle(N, nO, s["eHF"], E)
    de = torch.from_numpy(s["eHF"]).cuda()
    dL = torch.from_numpy(api.L_fortran_flat(s["L"])).cuda()
    ec_L = api.rpa_ecorr_quad_dev(N, 0, nO, 0, de.data_ptr(), d_L=dL.data_ptr(), naux=naux,
                                  ctx=ctx)
    assert ec_L is not None
    assert abs(ec_L - ref) < 1e-8 * max(1.0, abs(ref)), (ec_L, ref)
    dE = synth.eri_fortran_flat_torch(s["L"], device="cuda")
    ec_E = api.rpa_ecorr_quad_dev(N, 0, nO, 0, de.data_ptr(), d_ERI=dE.data_ptr(), ctx=ctx)
    nS = nO * (N - nO)
    if naux < nS // 3:
        assert ec_E is not None
        assert abs(ec_E - ref) < 1e-8 * max(1.0, abs(ref)), (ec_E, ref)
    else:
        assert ec_E is None  # (ia|jb) of numerical rank above nS/3: the eigenvalue route


def test_quadrature_negative_gap_is_nan_and_zero_gap_declines(ctx):
    """A virtual below an occupied orbital makes A - B indefinite: the Casida energy is NaN (the
    reference takes square roots of negative values) -- the quadrature says so without a
    factorisation; an exactly zero e_a - e_i is left to the eigenvalue route."""
    import torch
    N, nO, naux = 40, 5, 40
    s = synth.small_system(N, nO, naux, 36)
    dL = torch.from_numpy(api.L_fortran_flat(s["L"])).cuda()
    e = s["eHF"].copy()
    e[nO] = e[nO - 1] - 0.01
    de = torch.from_numpy(e).cuda()
    ec = api.rpa_ecorr_quad_dev(N, 0, nO, 0, de.data_ptr(), d_L=dL.data_ptr(), naux=naux, ctx=ctx)
    assert ec is not None and np.isnan(ec)
    e[nO] = e[nO - 1]
    de = torch.from_numpy(e).cuda()
    assert api.rpa_ecorr_quad_dev(N, 0, nO, 0, de.data_ptr(), d_L=dL.data_ptr(), naux=naux,
                                  ctx=ctx) is None


def test_mixed_g0w0_ecrpa_by_quadrature(ctx):
    """Mixed-tier drivers: the EcRPA at the G0W0 energies equals the Casida value at those
    energies (ERI driver with (ia|jb) of low rank, and the factorised driver)."""
    import torch
    N, nO, naux = 48, 6, 40
    s = synth.small_system(N, nO, naux, 35)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    r = api.RG0W0(api.GWOptions(precision=api.QK_PREC_BF16X3), N, N, 0, nO, N - nO, 0, nS, E,
                  s["eHF"], ctx=ctx)
    ref = _ec_oracle(N, nO, r["eGW"], E)
    assert abs(r["EcRPA"] - ref) < 1e-8 * max(1.0, abs(ref)), (r["EcRPA"], ref)
    dL = torch.from_numpy(api.L_fortran_flat(s["L"])).cuda()
    de = torch.from_numpy(s["eHF"]).cuda()
    out = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(3)]
    dOm = torch.empty(nS, dtype=torch.float64, device="cuda")
    ec, _ = api.RG0W0_L_dev(api.GWOptions(precision=api.QK_PREC_BF16X3), N, 0, nO, 0, naux,
                            dL.data_ptr(), de.data_ptr(), out[0].data_ptr(), out[1].data_ptr(),
                            out[2].data_ptr(), dOm.data_ptr(), ctx=ctx)
    refL = _ec_oracle(N, nO, out[0].cpu().numpy(), E)
    assert abs(ec - refL) < 1e-8 * max(1.0, abs(refL)), (ec, refL)
