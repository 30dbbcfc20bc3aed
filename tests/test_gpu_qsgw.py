"""GPU tests of quasiparticle self-consistent GW (GW/qsRGW.f90) against the oracle restatement:
He/6-31G and linear H chains in s-Gaussian bases (real AO integrals, non-orthogonal basis),
converged runs with and without DIIS, a fixed number of cycles of a run that does not converge
(the reference stops there), Tamm-Dancoff screening, the SRG-regularised self-energy, a frozen
core and virtual, fewer orbitals than basis functions, the device-pointer entry, and the mixed
precision tier.

Orbital coefficients are defined up to a sign per column, so the comparisons use the quantities
that do not depend on it: energies, eGW, the density matrix P and the diagonal of SigC."""
import numpy as np
import pytest

from oracle import he631g
from oracle import qkgw_oracle as O
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _he():
    S, T, V, eri = he631g.integrals()
    Hc = T + V
    E, eps, C = he631g.rhf(S, Hc, eri, 1)
    s, U = np.linalg.eigh(S)
    X = (U * s ** -0.5) @ U.T
    P = 2.0 * C[:, :1] @ C[:, :1].T
    return dict(nBas=2, nO=1, S=S, T=T, V=V, Hc=Hc, X=X, ERI_AO=eri, eHF=eps, cHF=C, PHF=P)


_CACHE = {}


def _chain(n_atoms, spacing=1.6, n_drop=0):
    key = (n_atoms, spacing, n_drop)
    if key not in _CACHE:
        _CACHE[key] = synth.hchain_system(n_atoms, spacing, n_drop=n_drop)
    return _CACHE[key]


def _run_both(ctx, sy, maxSCF=64, thresh=1e-5, max_diis=5, eta=0.05, TDA_W=False, doSRG=False,
              nC=0, nR=0, precision=api.QK_PREC_FP64, raise_on_fail=True):
    nb, nO = sy["nBas"], sy["nO"]
    n = sy.get("nOrb", nb)
    nS = (nO - nC) * (n - nO - nR)
    args = (nb, n, nC, nO, n - nO, nR, nS, sy["eHF"], sy["cHF"], sy["PHF"], sy["S"], sy["T"],
            sy["V"], sy["Hc"], sy["X"], sy["ERI_AO"])
    ref = O.qsRGW(maxSCF, thresh, max_diis, eta, TDA_W, *args, raise_on_fail=raise_on_fail,
                  doSRG=doSRG)
    opts = api.GWOptions(maxSCF=maxSCF, thresh=thresh, max_diis=max_diis, eta=eta, TDA_W=TDA_W,
                         reg=doSRG, precision=precision)
    got = api.qsRGW(opts, *args, ctx=ctx, raise_on_fail=raise_on_fail)
    return ref, got


def _compare(ref, got, tol):
    assert got["nSCF"] == ref["nSCF"]
    assert got["failed"] == ref["failed"]
    assert np.max(np.abs(got["eGW"] - ref["eGW"])) < tol
    assert np.max(np.abs(got["P"] - ref["P"])) < tol
    for k in ("EqsGW", "EcRPA", "EcGM"):
        assert abs(got[k] - ref[k]) < tol, k
    assert np.max(np.abs(got["Z"] - ref["Z"])) < tol
    assert np.max(np.abs(np.diag(got["SigC"]) - np.diag(ref["SigC"]))) < tol


def test_qsgw_he631g(ctx):
    ref, got = _run_both(ctx, _he(), eta=0.0)
    _compare(ref, got, 1e-9)
    assert not got["failed"] and got["Conv"] <= 1e-5


@pytest.mark.parametrize("n_atoms,eta,max_diis", [(4, 0.05, 5), (8, 0.01, 5), (6, 0.1, 1)])
def test_qsgw_hchain_converged(ctx, n_atoms, eta, max_diis):
    ref, got = _run_both(ctx, _chain(n_atoms), eta=eta, max_diis=max_diis, maxSCF=128)
    assert not ref["failed"]
    _compare(ref, got, 1e-8)
    assert abs(got["Conv"] - ref["Conv"]) < 1e-9


def test_qsgw_fixed_cycles_unconverged(ctx):
    """eta = 0 on H8: the run is stopped after maxSCF cycles and reported as not converged."""
    ref, got = _run_both(ctx, _chain(8), eta=0.0, maxSCF=4, raise_on_fail=False)
    assert ref["failed"] and got["failed"] and got["nSCF"] == 4
    _compare(ref, got, 1e-8)
    assert abs(got["Conv"] - ref["Conv"]) < 1e-9


def test_qsgw_tda_w_and_srg(ctx):
    ref, got = _run_both(ctx, _chain(6), eta=0.05, TDA_W=True)
    _compare(ref, got, 1e-8)
    ref, got = _run_both(ctx, _chain(6), eta=0.0, doSRG=True, maxSCF=6, raise_on_fail=False)
    _compare(ref, got, 1e-8)


def test_qsgw_frozen_core_and_virtual(ctx):
    ref, got = _run_both(ctx, _chain(6), eta=0.05, nC=1, nR=2)
    _compare(ref, got, 1e-8)


@pytest.mark.parametrize("n_atoms,n_drop", [(6, 1), (8, 3)])
def test_qsgw_fewer_orbitals_than_basis_functions(ctx, n_atoms, n_drop):
    """nOrb < nBas (canonical orthogonalisation without the smallest overlap eigenvalues): F is
    projected through c and Fp = c^T F c (qsRGW.f90:281-284, 328-333)."""
    sy = _chain(n_atoms, n_drop=n_drop)
    assert sy["nOrb"] == sy["nBas"] - n_drop
    ref, got = _run_both(ctx, sy, eta=0.05)
    assert not ref["failed"]
    _compare(ref, got, 1e-8)


def test_qsgw_device_entry_matches_host(ctx):
    torch = pytest.importorskip("torch")
    sy = _chain(4)
    n, nO = sy["nBas"], sy["nO"]
    opts = api.GWOptions(maxSCF=64, thresh=1e-5, max_diis=5, eta=0.05)
    host = api.qsRGW(opts, n, n, 0, nO, n - nO, 0, nO * (n - nO), sy["eHF"], sy["cHF"], sy["PHF"],
                     sy["S"], sy["T"], sy["V"], sy["Hc"], sy["X"], sy["ERI_AO"], ctx=ctx)

    def dev(a):  # column-major device copy
        return torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()

    d = {k: dev(sy[k]) for k in ("eHF", "cHF", "PHF", "S", "T", "V", "Hc", "X", "ERI_AO")}
    eGW = torch.empty(n, dtype=torch.float64, device="cuda")
    c = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P = torch.empty(n * n, dtype=torch.float64, device="cuda")
    Z = torch.empty(n, dtype=torch.float64, device="cuda")
    r = api.qsRGW_dev(opts, n, 0, nO, 0, *[d[k].data_ptr() for k in ("eHF", "cHF", "PHF", "S", "T",
                                                                      "V", "Hc", "X", "ERI_AO")],
                      eGW.data_ptr(), c.data_ptr(), P.data_ptr(), Z.data_ptr(), ctx=ctx)
    torch.cuda.synchronize()
    assert r["nSCF"] == host["nSCF"]
    assert np.max(np.abs(eGW.cpu().numpy() - host["eGW"])) < 1e-12
    assert np.max(np.abs(P.cpu().numpy().reshape(n, n, order="F") - host["P"])) < 1e-12
    assert abs(r["EqsGW"] - host["EqsGW"]) < 1e-12


def test_qsgw_mixed_tier_within_1meV(ctx):
    ref, got = _run_both(ctx, _chain(8), eta=0.01, precision=api.QK_PREC_BF16X3, maxSCF=128)
    assert not got["failed"]
    assert np.max(np.abs(got["eGW"] - ref["eGW"])) < 3.6749e-5   # 1 meV
    assert abs(got["EqsGW"] - ref["EqsGW"]) < 3.6749e-5


@pytest.mark.parametrize("srg", [False, True])
def test_full_self_energy_stage(ctx, srg):
    """Stage-level drop-in of RGW_self_energy / RGW_SRG_self_energy (unsymmetrised SigC)."""
    rng = np.random.default_rng(11)
    N, nO, nC, nR = 14, 4, 1, 2
    nS = (nO - nC) * (N - nO - nR)
    e = np.sort(rng.uniform(-3.0, 2.0, N))
    Om = np.sort(rng.uniform(0.2, 4.0, nS))
    rho = rng.standard_normal((N, N, nS)) * 0.3
    if srg:
        ref = O.RGW_SRG_self_energy(500.0, N, N, nC, nO, N - nO, nR, nS, e, Om, rho)
        got = api.RGW_self_energy(0.0, N, N, nC, nO, N - nO, nR, nS, e, Om, rho, ctx=ctx,
                                  srg_flow=500.0)
    else:
        ref = O.RGW_self_energy(0.02, N, N, nC, nO, N - nO, nR, nS, e, Om, rho)
        got = api.RGW_self_energy(0.02, N, N, nC, nO, N - nO, nR, nS, e, Om, rho, ctx=ctx)
    scale = max(1.0, np.max(np.abs(ref[1])))
    assert np.max(np.abs(got[1] - ref[1])) < 1e-11 * scale
    assert np.max(np.abs(got[2] - ref[2])) < 1e-11
    assert abs(got[0] - ref[0]) < 1e-11 * max(1.0, abs(ref[0]))


def test_hartree_exchange_stage(ctx):
    """Hartree_matrix_AO_basis / exchange_matrix_AO_basis on an H-chain density and on a
    tensor without any permutational symmetry (the kernel reads the indices as written)."""
    sy = _chain(4)
    n = sy["nBas"]
    for E, P in ((sy["ERI_AO"], sy["PHF"]),
                 (np.random.default_rng(5).standard_normal((n,) * 4),
                  np.random.default_rng(6).standard_normal((n, n)))):
        H = api.Hartree_matrix_AO_basis(n, P, E, ctx=ctx)
        K = api.exchange_matrix_AO_basis(n, P, E, ctx=ctx)
        assert np.max(np.abs(H - O.Hartree_matrix_AO_basis(n, P, E))) < 1e-12 * max(1, np.abs(H).max())
        assert np.max(np.abs(K - O.exchange_matrix_AO_basis(n, P, E))) < 1e-12 * max(1, np.abs(K).max())


def test_qsgw_argument_errors_and_single_cycle(ctx):
    """max_diis above the DIIS kernel's 32, nBas < nOrb and negative maxSCF are refused; maxSCF = 0
    runs exactly one cycle and, as in the reference (nSCF == maxSCF), reports no convergence."""
    sy = _chain(4)
    n, nO = sy["nBas"], sy["nO"]
    args = (n, n, 0, nO, n - nO, 0, nO * (n - nO), sy["eHF"], sy["cHF"], sy["PHF"], sy["S"],
            sy["T"], sy["V"], sy["Hc"], sy["X"], sy["ERI_AO"])
    for opts in (api.GWOptions(max_diis=40, eta=0.05), api.GWOptions(maxSCF=-1, eta=0.05)):
        with pytest.raises(api.QkError):
            api.qsRGW(opts, *args, ctx=ctx)
    bad = (n - 1,) + args[1:]
    with pytest.raises(api.QkError):
        api.qsRGW(api.GWOptions(eta=0.05), *bad, ctx=ctx)
    got = api.qsRGW(api.GWOptions(maxSCF=0, eta=0.05, max_diis=5), *args, ctx=ctx,
                    raise_on_fail=False)
    ref = O.qsRGW(0, 1e-5, 5, 0.05, False, *args, raise_on_fail=False)
    assert got["failed"] and ref["failed"] and got["nSCF"] == 0 == ref["nSCF"]
    _compare(ref, got, 1e-9)
    # the context stays usable after the refused calls
    ref, got = _run_both(ctx, sy, eta=0.05)
    _compare(ref, got, 1e-8)
