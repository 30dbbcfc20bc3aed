"""CPU tests: pin the oracle to the reference's golden values and known answers.

He/6-31G values: FeatherBench (reference tests/feather_bench.py:62-91); the reference bench
compares at relative 1e-7 by default (tests/lunch_bench.py:62-69).  The evGW goldens are
reproduced with the DIIS extrapolation off (max_diis = 1); with DIIS = 5, as in
tests/inp/options.RHF, evRGW.f90 as written follows a different trajectory that stops
2.9e-7 Ha away (still inside its 1e-5 convergence threshold), so the goldens were evidently
produced without DIIS.
"""
import os

import numpy as np
import pytest

from oracle import qkgw_oracle as O
from oracle.he631g import GOLDEN, he_system
from quack_gb300 import synth

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def he():
    return he_system()


def test_he_rhf_matches_featherbench(he):
    assert abs(he["ERHF"] - GOLDEN["RHF energy"]) < 1e-10
    assert abs(he["eHF"][0] - GOLDEN["RHF HOMO energy"]) < 1e-9
    assert abs(he["eHF"][1] - GOLDEN["RHF LUMO energy"]) < 1e-9


def test_he_g0w0_matches_featherbench(he):
    r = O.RG0W0(False, 0.0, False, 2, 2, 0, 1, 1, 0, 1, he["ERI_MO"], he["eHF"])
    assert abs(r["EcRPA"] - GOLDEN["G0W0 correlation energy"]) < 1e-10
    assert abs(r["eGW"][0] - GOLDEN["G0W0 HOMO energy"]) < 1e-10
    assert abs(r["eGW"][1] - GOLDEN["G0W0 LUMO energy"]) < 1e-10
    assert abs(r["EcRPA_HF"] - GOLDEN["phRPA correlation energy"]) < 1e-10


def test_he_evgw_matches_featherbench_without_diis(he):
    r = O.evRGW(256, 1e-5, 1, False, 0.0, False, 2, 2, 0, 1, 1, 0, 1, he["ERI_MO"], he["eHF"])
    assert abs(r["EcRPA"] - GOLDEN["evGW correlation energy"]) < 1e-10
    assert abs(r["eGW"][0] - GOLDEN["evGW HOMO energy"]) < 1e-10
    assert abs(r["eGW"][1] - GOLDEN["evGW LUMO energy"]) < 1e-10


def test_he_evgw_with_diis_within_threshold(he):
    r = O.evRGW(256, 1e-5, 5, False, 0.0, False, 2, 2, 0, 1, 1, 0, 1, he["ERI_MO"], he["eHF"])
    assert abs(r["eGW"][0] - GOLDEN["evGW HOMO energy"]) < 1e-5
    assert r["nSCF"] == 3


def test_he_cis_matches_reference_test_data(he):
    """The non-dRPA ph blocks that the BSE builds on: CIS = TDA of phRLR_A(ispin, dRPA=False) at
    eHF, against the reference's own test data (test/Rtest_ref.dat:27-30, He/6-31G; its RHF energy
    there differs from FeatherBench's by 7e-10 Ha, hence the 1e-8 bar)."""
    E, e = he["ERI_MO"], he["eHF"]
    for ispin, ref in ((1, 1.911193619935257), (2, 1.455852629402236)):
        A = O.phRLR_A(ispin, False, 2, 0, 1, 1, 0, 1, 1.0, e, E)
        _, Om, _, _ = O.phRLR(True, 1, A, np.zeros((1, 1)))
        assert abs(Om[0] - ref) < 1e-8, (ispin, Om[0], ref)


def test_bse_static_kernels_match_reference_loops():
    """The einsum form of RGW_phBSE_static_kernel_A/B against the reference's loop nest
    (GW/RGW_phBSE_static_kernel_A.f90:32-52, _B.f90:32-52) on a small random rho with a frozen
    core and a frozen virtual."""
    rng = np.random.default_rng(5)
    N, nC, nO, nR = 9, 1, 4, 1
    no, nv = nO - nC, N - nO - nR
    nS = no * nv
    rho = rng.standard_normal((N, N, nS))
    Om = np.sort(rng.uniform(0.2, 3.0, nS))
    eta = 0.05
    KA = O.RGW_phBSE_static_kernel_A(eta, N, nC, nO, N - nO, nR, nS, 1.0, Om, rho)
    KB = O.RGW_phBSE_static_kernel_B(eta, N, nC, nO, N - nO, nR, nS, 1.0, Om, rho)
    ia = 0
    for i in range(nC, nO):
        for a in range(nO, N - nR):
            jb = 0
            for j in range(nC, nO):
                for b in range(nO, N - nR):
                    ca = sum(rho[i, j, k] * rho[a, b, k] * Om[k] / (Om[k] ** 2 + eta ** 2)
                             for k in range(nS))
                    cb = sum(rho[i, b, k] * rho[a, j, k] * Om[k] / (Om[k] ** 2 + eta ** 2)
                             for k in range(nS))
                    assert abs(KA[ia, jb] - 4.0 * ca) < 1e-12 * max(1.0, abs(ca))
                    assert abs(KB[ia, jb] - 4.0 * cb) < 1e-12 * max(1.0, abs(cb))
                    jb += 1
            ia += 1


def test_casida_closed_form_ns1(he):
    """nS = 1: Omega = sqrt(Delta (Delta + 4 (ia|ia)))."""
    E, e = he["ERI_MO"], he["eHF"]
    A = O.phRLR_A(1, True, 2, 0, 1, 1, 0, 1, 1.0, e, E)
    B = O.phRLR_B(1, True, 2, 0, 1, 1, 0, 1, 1.0, E)
    Ec, Om, XpY, XmY = O.phRLR(False, 1, A, B)
    d = e[1] - e[0]
    K = E[1, 0, 0, 1]
    assert abs(Om[0] - np.sqrt(d * (d + 4 * K))) < 1e-13
    assert abs(Ec - 0.5 * (Om[0] - A[0, 0])) < 1e-15


def test_ecrpa_identity_and_orthogonality():
    s = synth.small_system(12, 3, 36, 5)
    E = synth.eri_phys_numpy(s["L"])
    nS = 3 * 9
    A = O.phRLR_A(1, True, 12, 0, 3, 9, 0, nS, 1.0, s["eHF"], E)
    B = O.phRLR_B(1, True, 12, 0, 3, 9, 0, nS, 1.0, E)
    Ec, Om, XpY, XmY = O.phRLR(False, nS, A, B)
    assert abs(Ec - 0.5 * (Om.sum() - np.trace(A))) < 1e-12
    # (X+Y)^T (X-Y) = 1 (Casida normalisation)
    assert np.allclose(XpY @ XmY.T, np.eye(nS), atol=1e-10)
    # A+B and A-B positive definite for the synthetic generator
    assert np.linalg.eigvalsh(A + B).min() > 0 and np.linalg.eigvalsh(A - B).min() > 0


def test_eri_symmetry_of_generator():
    s = synth.small_system(7, 2, 21, 3)
    E = synth.eri_phys_numpy(s["L"])
    # <pq|rs> = <qp|sr> = <rq|ps> = <ps|rq> ... 8-fold for real orbitals
    assert np.allclose(E, E.transpose(1, 0, 3, 2))
    assert np.allclose(E, E.transpose(2, 1, 0, 3))
    assert np.allclose(E, E.transpose(0, 3, 2, 1))
    assert np.allclose(E, E.transpose(2, 3, 0, 1))


def test_excitation_density_identity():
    """rho with XpY = identity equals the ERI slab (pq|jb)."""
    s = synth.small_system(8, 2, 24, 4)
    E = synth.eri_phys_numpy(s["L"])
    nS = 2 * 6
    rho = O.RGW_excitation_density(8, 0, 2, 0, nS, E, np.eye(nS))
    for j in range(2):
        for b in range(6):
            assert np.allclose(rho[:, :, j * 6 + b], E[:, j, :, 2 + b])


def test_sigma_invariant_under_sign_flips():
    s = synth.small_system(10, 2, 30, 6)
    E = synth.eri_phys_numpy(s["L"])
    nS = 16
    A = O.phRLR_A(1, True, 10, 0, 2, 8, 0, nS, 1.0, s["eHF"], E)
    B = O.phRLR_B(1, True, 10, 0, 2, 8, 0, nS, 1.0, E)
    _, Om, XpY, _ = O.phRLR(False, nS, A, B)
    rng = np.random.default_rng(0)
    sg = rng.choice([-1.0, 1.0], size=nS)
    r1 = O.RGW_excitation_density(10, 0, 2, 0, nS, E, XpY)
    r2 = O.RGW_excitation_density(10, 0, 2, 0, nS, E, sg[:, None] * XpY)
    s1 = O.RGW_self_energy_diag(0.0, 10, 10, 0, 2, 8, 0, nS, s["eHF"], Om, r1)
    s2 = O.RGW_self_energy_diag(0.0, 10, 10, 0, 2, 8, 0, nS, s["eHF"], Om, r2)
    assert np.allclose(s1[1], s2[1], rtol=1e-12, atol=1e-14)
    assert abs(s1[0] - s2[0]) < 1e-12


def test_aotomo_matches_einsum():
    rng = np.random.default_rng(1)
    nB, nO_ = 5, 4
    ERI = rng.standard_normal((nB,) * 4)
    c = rng.standard_normal((nB, nO_))
    ref = np.einsum("abcd,ap,bq,cr,ds->pqrs", ERI, c, c, c, c)
    assert np.allclose(O.AOtoMO_ERI_RHF(nB, nO_, c, ERI), ref)


def test_diis_against_closed_form():
    """Two-vector DIIS: weights minimise |w1 r1 + w2 r2| with w1 + w2 = 1."""
    n = 4
    rng = np.random.default_rng(2)
    r1, r2 = rng.standard_normal(n), rng.standard_normal(n)
    e1, e2 = rng.standard_normal(n), rng.standard_normal(n)
    err = np.zeros((n, 3), order="F")
    ee = np.zeros((n, 3), order="F")
    _, err, ee, out = O.DIIS_extrapolation(1, err, ee, r1, e1)
    assert np.allclose(out, e1)
    rc, err, ee, out = O.DIIS_extrapolation(2, err, ee, r2, e2)
    d = r2 - r1
    w2 = -(r1 @ d) / (d @ d)
    assert np.allclose(out, (1 - w2) * e1 + w2 * e2)
    assert rc > 1e-13


def test_fixtures_reproduce_with_oracle():
    """The committed fixtures are what the oracle computes now (guards accidental edits)."""
    for name in ("synth_n24", "synth_n13_frozen"):
        f = np.load(os.path.join(GOLD, name + ".npz"))
        N, nO, nC, nR = int(f["N"]), int(f["nO"]), int(f["nC"]), int(f["nR"])
        E = synth.eri_phys_numpy(f["L"])
        nS = (nO - nC) * (N - nO - nR)
        r = O.RG0W0(False, 0.0, False, N, N, nC, nO, N - nO, nR, nS, E, f["eHF"])
        assert np.allclose(r["eGW"], f["g0w0_eGW"], atol=1e-11)
        assert abs(r["EcRPA"] - float(f["g0w0_EcRPA"])) < 1e-11


def test_generator_is_deterministic():
    a = synth.small_system(9, 2, 27, 123)
    b = synth.small_system(9, 2, 27, 123)
    assert np.array_equal(a["L"], b["L"]) and np.array_equal(a["eHF"], b["eHF"])
    assert synth.n_occ(20) == 3 and synth.n_occ(24) == 3 and synth.n_occ(28) == 4


# ---------------------------------------------------------------------------------------------
# quasiparticle self-consistent GW (GW/qsRGW.f90): the reference ships no qsGW golden numbers, so
# the restatement is tied to the pinned pieces it is built from
# ---------------------------------------------------------------------------------------------
def test_qsgw_full_self_energy_diagonal_is_the_pinned_diagonal():
    """RGW_self_energy's diagonal, Z and EcGM equal RGW_self_energy_diag's (pinned by the G0W0
    goldens); the same for the SRG forms."""
    rng = np.random.default_rng(7)
    N, nO, nC, nR = 9, 3, 1, 1
    nS = (nO - nC) * (N - nO - nR)
    e = np.sort(rng.uniform(-2.0, 2.0, N))
    Om = np.sort(rng.uniform(0.3, 3.0, nS))
    rho = rng.standard_normal((N, N, nS)) * 0.2
    for full, diag, arg in ((O.RGW_self_energy, O.RGW_self_energy_diag, 0.03),
                            (O.RGW_SRG_self_energy, O.RGW_SRG_self_energy_diag, 500.0)):
        Ec1, Sig, Z1 = full(arg, N, N, nC, nO, N - nO, nR, nS, e, Om, rho)
        Ec2, sd, Z2 = diag(arg, N, N, nC, nO, N - nO, nR, nS, e, Om, rho)
        assert np.max(np.abs(np.diag(Sig) - sd)) < 1e-13
        assert np.max(np.abs(Z1 - Z2)) < 1e-13 and abs(Ec1 - Ec2) < 1e-13
        assert np.all(Sig[:nC] == 0.0) and np.all(Sig[:, N - nR:] == 0.0)


def test_qsgw_hf_energy_terms_reproduce_rhf():
    """At the RHF density, ET + EV + EJ + EK of the qsGW loop is the RHF electronic energy."""
    from oracle import he631g
    S, T, V, eri = he631g.integrals()
    E, eps, C = he631g.rhf(S, T + V, eri, 1)
    P = 2.0 * C[:, :1] @ C[:, :1].T
    J = O.Hartree_matrix_AO_basis(2, P, eri)
    K = O.exchange_matrix_AO_basis(2, P, eri)
    Eq = (O.trace_matrix(P @ T) + O.trace_matrix(P @ V) + 0.5 * O.trace_matrix(P @ J)
          + 0.25 * O.trace_matrix(P @ K))
    assert abs(Eq - E) < 1e-10
    # MOtoAO and AOtoMO are inverse to each other when c^T S c = 1
    M = np.array([[0.3, -0.1], [-0.1, 0.7]])
    assert np.max(np.abs(O.AOtoMO(2, 2, C, O.MOtoAO(2, 2, S, C, M)) - M)) < 1e-12


def test_qsgw_oracle_converges_on_h4():
    from quack_gb300 import synth
    sy = synth.hchain_system(4)
    n, nO = sy["nBas"], sy["nO"]
    r = O.qsRGW(64, 1e-5, 5, 0.05, False, n, n, 0, nO, n - nO, 0, nO * (n - nO), sy["eHF"],
                sy["cHF"], sy["PHF"], sy["S"], sy["T"], sy["V"], sy["Hc"], sy["X"], sy["ERI_AO"])
    assert not r["failed"] and r["Conv"] <= 1e-5
    # qsGW moves the RHF energy by a few mHa
    assert abs(r["EqsGW"] - sy["ERHF"]) < 1e-2
    c = r["c"]
    assert np.max(np.abs(c.T @ sy["S"] @ c - np.eye(n))) < 1e-10


def test_acfdt_correlation_energy_matrices_follow_the_loops():
    """The vectorised Ap/Bp of phACFDT_correlation_energy against the reference's index loops
    (RPA/phACFDT_correlation_energy.f90:56-70) on a tensor without symmetry."""
    rng = np.random.default_rng(3)
    N, nC, nO, nR = 7, 1, 3, 1
    nV = N - nO
    nS = (nO - nC) * (N - nO - nR)
    E = rng.standard_normal((N,) * 4)
    XpY = rng.standard_normal((nS, nS))
    XmY = rng.standard_normal((nS, nS))
    for ispin in (1, 2):
        for xk in (False, True):
            ds = 1.0 if ispin == 1 else -1.0
            dK = 1.0 if xk else 0.0
            Ap = np.zeros((nS, nS))
            Bp = np.zeros((nS, nS))
            ia = 0
            for i in range(nC, nO):
                for a in range(nO, N - nR):
                    jb = 0
                    for j in range(nC, nO):
                        for b in range(nO, N - nR):
                            Ap[ia, jb] = (1 + ds) * E[i, b, a, j] - dK * E[i, b, j, a]
                            Bp[ia, jb] = (1 + ds) * E[i, j, a, b] - dK * E[i, j, b, a]
                            jb += 1
                    ia += 1
            X, Y = 0.5 * (XpY + XmY), 0.5 * (XpY - XmY)
            ref = (np.trace(X @ Bp @ Y.T + Y @ Bp @ X.T) + np.trace(X @ Ap @ X.T + Y @ Ap @ Y.T)
                   - np.trace(Ap))
            got = O.phACFDT_correlation_energy(ispin, xk, N, nC, nO, nV, nR, nS, E, XpY, XmY)
            assert abs(got - ref) < 1e-10 * max(1.0, abs(ref))


def test_hchain_integrals_are_those_of_real_gaussians():
    """The closed-form s-Gaussian integrals of the H-chain inputs: normalised primitives
    (S_ii = 1), symmetric positive-definite S, T, the 8-fold permutational symmetry of the
    physicist ERI tensor, the positive-semidefinite (pq|rs) supermatrix, the nuclear repulsion,
    and the one-centre closed forms."""
    from quack_gb300 import synth
    S, T, V, E, ENuc = synth.hchain_integrals(4, 1.6)
    n = S.shape[0]
    assert np.allclose(np.diag(S), 1.0, atol=1e-14)
    for M in (S, T, V):
        assert np.max(np.abs(M - M.T)) < 1e-14
    assert np.linalg.eigvalsh(S).min() > 0 and np.linalg.eigvalsh(T).min() > 0
    for perm in ((1, 0, 3, 2), (2, 1, 0, 3), (0, 3, 2, 1), (2, 3, 0, 1)):
        assert np.max(np.abs(E - E.transpose(perm))) < 1e-13
    chem = E.transpose(0, 2, 1, 3).reshape(n * n, n * n)
    assert np.linalg.eigvalsh(chem).min() > -1e-12
    assert abs(ENuc - sum(1.0 / (1.6 * abs(i - j)) for i in range(4) for j in range(i))) < 1e-14
    # one normalised primitive (the partner atom 50 bohr away): <aa|aa> by the one-centre
    # formula 2 pi^2.5 / (p q sqrt(p + q)) N^4 with p = q = 2a, and <a|T|a> = 3a/2
    a = synth.HCHAIN_EXPONENTS[0]
    S1, T1, V1, E1, _ = synth.hchain_integrals(2, 50.0, exponents=(a,))
    nrm = (2 * a / np.pi) ** 0.75
    p = 2 * a
    assert abs(E1[0, 0, 0, 0] - 2 * np.pi ** 2.5 / (p * p * np.sqrt(2 * p)) * nrm ** 4) < 1e-12
    assert abs(T1[0, 0] - 1.5 * a) < 1e-12


def test_qsgw_oracle_invariances():
    """Properties of the qsGW restatement: the result does not depend on the signs of the
    starting orbitals, nor on which orthogonaliser X spans the basis (symmetric S^-1/2 or
    canonical U s^-1/2), and the converged Fock matrix commutes with P S to the threshold."""
    from quack_gb300 import synth
    sy = synth.hchain_system(4)
    n, nO = sy["nBas"], sy["nO"]
    args = (n, n, 0, nO, n - nO, 0, nO * (n - nO))

    def run(c, X):
        return O.qsRGW(64, 1e-7, 5, 0.05, False, *args, sy["eHF"], c, sy["PHF"], sy["S"], sy["T"],
                       sy["V"], sy["Hc"], X, sy["ERI_AO"])

    ref = run(sy["cHF"], sy["X"])
    signs = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
    flipped = run(sy["cHF"] * signs[None, :], sy["X"])
    s, U = np.linalg.eigh(sy["S"])
    canon = run(sy["cHF"], U * s ** -0.5)
    for r in (flipped, canon):
        assert np.max(np.abs(r["eGW"] - ref["eGW"])) < 1e-7
        assert np.max(np.abs(r["P"] - ref["P"])) < 1e-6
        assert abs(r["EqsGW"] - ref["EqsGW"]) < 1e-8
    assert not ref["failed"] and ref["Conv"] <= 1e-7


def test_qp_graph_maxit_fallback():
    """RGW_QP_graph.f90:78-81: a search that reaches maxIt keeps eGWlin and Z; the test is
    nIt == maxIt after the loop, so it applies even when the last step met the threshold."""
    from oracle import qkgw_oracle as O
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = int(f["N"]), int(f["nO"])
    nS = nO * (N - nO)
    E = synth.eri_phys_numpy(f["L"])
    ref = O.RG0W0(True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, f["eHF"])
    Z0 = ref["Z"]
    full = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, f["eHF"], ref["Om"],
                          ref["rho"], ref["eGWlin"], f["eHF"], Z0, return_iters=True)
    assert np.max(np.abs(full[0] - f["g0w0_eGW"])) < 1e-12
    for mi in (1, int(full[2].max())):
        eGW, Z, it = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, f["eHF"],
                                    ref["Om"], ref["rho"], ref["eGWlin"], f["eHF"], Z0,
                                    return_iters=True, maxit=mi)
        hit = it == mi
        assert hit.any()
        assert np.array_equal(eGW[hit], ref["eGWlin"][hit])
        assert np.array_equal(Z[hit], Z0[hit])
        assert np.array_equal(eGW[~hit], full[0][~hit])


def test_qp_root_certificate_implies_reference_root():
    """Whenever the root certificate holds for a root r reached from another start, the
    reference Newton search from eGWlin (RGW_QP_graph.f90:56-76) ends on r."""
    from oracle import qkgw_oracle as O
    n_cert = 0
    for N, nO, seed in ((24, 3, 41), (32, 4, 42), (40, 5, 43)):
        s = synth.small_system(N, nO, 3 * N, seed)
        E = synth.eri_phys_numpy(s["L"])
        nS = nO * (N - nO)
        g = O.RG0W0(True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
        e, Om, rho, lin = s["eHF"], g["Om"], g["rho"], g["eGWlin"]
        rng = np.random.default_rng(seed)
        for p in range(N):
            for shift in rng.normal(0.0, 0.05, 3):
                # a root reached from a perturbed start
                w, f, it = lin[p] + shift, 1.0, 0
                while abs(f) > O.QP_THRESH and it < O.QP_MAXIT:
                    it += 1
                    f = w - e[p] - O.RGW_Re_SigC(p, w, 0.0, N, 0, nO, N - nO, 0, nS, e, Om, rho)
                    w -= f / (1.0 - O.RGW_Re_dSigC(p, w, 0.0, N, 0, nO, N - nO, 0, nS, e, Om, rho))
                if it == O.QP_MAXIT or not O.qp_root_certificate(p, w, lin[p], N, 0, nO, 0, e,
                                                                   Om, rho):
                    continue
                n_cert += 1
                ref, _ = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, e, Om, rho,
                                        lin, e, g["Z"])
                assert abs(ref[p] - w) < 1e-8, (N, p, ref[p], w)
    assert n_cert > 50
