! qk_gw_module.f90 -- Fortran bind(C) interfaces to libqkgw.so (include/qkgw.h).
!
! Same conventions as QuAcK's src/GPU/cu_quack_module.f90:11-36: integer(c_int) by value,
! real(c_double) arrays with explicit shape (passed as the first element, Fortran column-major).
! Every function returns an integer(c_int) status (0 = success).  The context is a type(c_ptr)
! obtained once from qk_init.
!
! Source only: no Fortran compiler is available where this library is built; the interfaces
! are checked against the C header by hand and the ABI itself is exercised from C/Python.
module qk_gw_module

  use, intrinsic :: iso_c_binding

  implicit none

  type, bind(C) :: qk_gw_params
    real(c_double)    :: eta
    integer(c_int)    :: linearize
    integer(c_int)    :: doSRG
    integer(c_int)    :: TDA_W
    integer(c_int)    :: maxSCF
    real(c_double)    :: thresh
    integer(c_int)    :: max_diis
    integer(c_int)    :: precision
    integer(c_int)    :: qp_guess
  end type qk_gw_params

  type, bind(C) :: qk_bse_params
    integer(c_int)    :: TDA_W
    integer(c_int)    :: TDA
    integer(c_int)    :: singlet
    integer(c_int)    :: triplet
    integer(c_int)    :: exchange_kernel
    real(c_double)    :: eta
  end type qk_bse_params

  integer(c_int), parameter :: QK_OK = 0, QK_ERR_NO_CONV = 5
  integer(c_int), parameter :: QK_PREC_FP64 = 0, QK_PREC_BF16X3 = 1

  interface

    integer(c_int) function qk_init(device, ctx) bind(C, name="qk_init")
      import c_int, c_ptr
      integer(c_int), value :: device
      type(c_ptr)           :: ctx
    end function qk_init

    integer(c_int) function qk_finalize(ctx) bind(C, name="qk_finalize")
      import c_int, c_ptr
      type(c_ptr), value :: ctx
    end function qk_finalize

    ! LR/phRLR_A.f90
    integer(c_int) function qk_phRLR_A(ctx, ispin, dRPA, nBas, nC, nO, nV, nR, nS, lambda, e, ERI, Aph) &
        bind(C, name="qk_phRLR_A")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: ispin, dRPA, nBas, nC, nO, nV, nR, nS
      real(c_double), value         :: lambda
      real(c_double), intent(in)    :: e(nBas), ERI(nBas,nBas,nBas,nBas)
      real(c_double), intent(out)   :: Aph(nS,nS)
    end function qk_phRLR_A

    ! LR/phRLR_B.f90
    integer(c_int) function qk_phRLR_B(ctx, ispin, dRPA, nBas, nC, nO, nV, nR, nS, lambda, ERI, Bph) &
        bind(C, name="qk_phRLR_B")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: ispin, dRPA, nBas, nC, nO, nV, nR, nS
      real(c_double), value         :: lambda
      real(c_double), intent(in)    :: ERI(nBas,nBas,nBas,nBas)
      real(c_double), intent(out)   :: Bph(nS,nS)
    end function qk_phRLR_B

    ! LR/phRLR.f90 (TDA must be 0)
    integer(c_int) function qk_phRLR(ctx, TDA, nS, Aph, Bph, EcRPA, Om, XpY, XmY) bind(C, name="qk_phRLR")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: TDA, nS
      real(c_double), intent(in)    :: Aph(nS,nS), Bph(nS,nS)
      real(c_double), intent(out)   :: EcRPA, Om(nS), XpY(nS,nS), XmY(nS,nS)
    end function qk_phRLR

    ! GW/RGW_excitation_density.f90
    integer(c_int) function qk_RGW_excitation_density(ctx, nOrb, nC, nO, nR, nS, ERI, XpY, rho) &
        bind(C, name="qk_RGW_excitation_density")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: nOrb, nC, nO, nR, nS
      real(c_double), intent(in)    :: ERI(nOrb,nOrb,nOrb,nOrb), XpY(nS,nS)
      real(c_double), intent(out)   :: rho(nOrb,nOrb,nS)
    end function qk_RGW_excitation_density

    ! GW/RGW_self_energy_diag.f90
    integer(c_int) function qk_RGW_self_energy_diag(ctx, eta, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho, &
        EcGM, Sig, Z) bind(C, name="qk_RGW_self_energy_diag")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      real(c_double), value         :: eta
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: e(nBas), Om(nS), rho(nBas,nBas,nS)
      real(c_double), intent(out)   :: EcGM, Sig(nBas), Z(nBas)
    end function qk_RGW_self_energy_diag

    integer(c_int) function qk_RGW_SRG_self_energy_diag(ctx, flow, nBas, nOrb, nC, nO, nV, nR, nS, e, &
        Om, rho, EcGM, Sig, Z) bind(C, name="qk_RGW_SRG_self_energy_diag")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      real(c_double), value         :: flow
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: e(nBas), Om(nS), rho(nBas,nBas,nS)
      real(c_double), intent(out)   :: EcGM, Sig(nBas), Z(nBas)
    end function qk_RGW_SRG_self_energy_diag

    ! utils/DIIS_extrapolation.f90 (error and e histories updated in place)
    integer(c_int) function qk_DIIS_extrapolation(ctx, rcond, n_err, n_e, n_diis, error, e, &
        error_in, e_inout) bind(C, name="qk_DIIS_extrapolation")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      real(c_double), intent(out)   :: rcond
      integer(c_int), value         :: n_err, n_e, n_diis
      real(c_double), intent(inout) :: error(n_err,*), e(n_e,*)
      real(c_double), intent(in)    :: error_in(n_err)
      real(c_double), intent(inout) :: e_inout(n_e)
    end function qk_DIIS_extrapolation

    ! precision tier of the stage-level drop-ins (QK_PREC_FP64 or QK_PREC_BF16X3)
    integer(c_int) function qk_set_stage_precision(ctx, precision) &
        bind(C, name="qk_set_stage_precision")
      import c_int, c_ptr
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: precision
    end function qk_set_stage_precision

    ! GW/RGW_QP_graph.f90 (Z is in/out, as in the reference)
    integer(c_int) function qk_RGW_QP_graph(ctx, doSRG, eta, flow, nBas, nC, nO, nV, nR, nS, eHF, Om, rho, &
        eGWlin, eOld, eGW, Z) bind(C, name="qk_RGW_QP_graph")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: doSRG, nBas, nC, nO, nV, nR, nS
      real(c_double), value         :: eta, flow
      real(c_double), intent(in)    :: eHF(nBas), Om(nS), rho(nBas,nBas,nS), eGWlin(nBas), eOld(nBas)
      real(c_double), intent(out)   :: eGW(nBas)
      real(c_double), intent(inout) :: Z(nBas)
    end function qk_RGW_QP_graph

    ! AOtoMO/AOtoMO_ERI_RHF.f90
    integer(c_int) function qk_AOtoMO_ERI_RHF(ctx, nBas, nOrb, c, ERI_AO, ERI_MO) bind(C, name="qk_AOtoMO_ERI_RHF")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: nBas, nOrb
      real(c_double), intent(in)    :: c(nBas,nOrb), ERI_AO(nBas,nBas,nBas,nBas)
      real(c_double), intent(out)   :: ERI_MO(nOrb,nOrb,nOrb,nOrb)
    end function qk_AOtoMO_ERI_RHF

    ! GW/RG0W0.f90 (driver)
    integer(c_int) function qk_RG0W0(ctx, prm, nBas, nOrb, nC, nO, nV, nR, nS, eHF, ERI, eGW, SigC, Z, Om, &
        EcRPA, EcGM) bind(C, name="qk_RG0W0")
      import c_int, c_ptr, c_double, qk_gw_params
      type(c_ptr), value            :: ctx
      type(qk_gw_params), intent(in):: prm
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: eHF(nOrb), ERI(nOrb,nOrb,nOrb,nOrb)
      real(c_double), intent(out)   :: eGW(nOrb), SigC(nOrb), Z(nOrb), Om(nS), EcRPA, EcGM
    end function qk_RG0W0

    ! GW/evRGW.f90 (driver; returns QK_ERR_NO_CONV where the reference stops)
    integer(c_int) function qk_evRGW(ctx, prm, nBas, nOrb, nC, nO, nV, nR, nS, eHF, ERI, eGW, SigC, Z, &
        EcRPA, EcGM, nSCF, Conv) bind(C, name="qk_evRGW")
      import c_int, c_ptr, c_double, qk_gw_params
      type(c_ptr), value            :: ctx
      type(qk_gw_params), intent(in):: prm
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: eHF(nOrb), ERI(nOrb,nOrb,nOrb,nOrb)
      real(c_double), intent(out)   :: eGW(nOrb), SigC(nOrb), Z(nOrb), EcRPA, EcGM, Conv
      integer(c_int), intent(out)   :: nSCF
    end function qk_evRGW

    integer(c_int) function qk_RGW_phBSE(ctx, prm, nBas, nOrb, nC, nO, nV, nR, nS, ERI, eW, eGW, &
        EcBSE, OmS, OmT) bind(C, name="qk_RGW_phBSE")
      import c_int, c_ptr, c_double, qk_bse_params
      type(c_ptr), value            :: ctx
      type(qk_bse_params), intent(in) :: prm
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: ERI(nOrb,nOrb,nOrb,nOrb), eW(nOrb), eGW(nOrb)
      real(c_double), intent(out)   :: EcBSE(2), OmS(nS), OmT(nS)
    end function qk_RGW_phBSE

    integer(c_int) function qk_RGW_phACFDT(ctx, prm, doXBS, nBas, nOrb, nC, nO, nV, nR, nS, ERI, &
        eW, eGW, EcAC) bind(C, name="qk_RGW_phACFDT")
      import c_int, c_ptr, c_double, qk_bse_params
      type(c_ptr), value            :: ctx
      type(qk_bse_params), intent(in) :: prm
      integer(c_int), value         :: doXBS, nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: ERI(nOrb,nOrb,nOrb,nOrb), eW(nOrb), eGW(nOrb)
      real(c_double), intent(out)   :: EcAC(2)
    end function qk_RGW_phACFDT

    integer(c_int) function qk_RGW_self_energy(ctx, eta, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, &
        rho, EcGM, SigC, Z) bind(C, name="qk_RGW_self_energy")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      real(c_double), value         :: eta
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: e(nOrb), Om(nS), rho(nOrb,nOrb,nS)
      real(c_double), intent(out)   :: EcGM, SigC(nOrb,nOrb), Z(nOrb)
    end function qk_RGW_self_energy

    integer(c_int) function qk_RGW_SRG_self_energy(ctx, flow, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, &
        rho, EcGM, SigC, Z) bind(C, name="qk_RGW_SRG_self_energy")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      real(c_double), value         :: flow
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: e(nOrb), Om(nS), rho(nOrb,nOrb,nS)
      real(c_double), intent(out)   :: EcGM, SigC(nOrb,nOrb), Z(nOrb)
    end function qk_RGW_SRG_self_energy

    integer(c_int) function qk_Hartree_matrix_AO_basis(ctx, nBas, P, ERI, H) &
        bind(C, name="qk_Hartree_matrix_AO_basis")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: nBas
      real(c_double), intent(in)    :: P(nBas,nBas), ERI(nBas,nBas,nBas,nBas)
      real(c_double), intent(out)   :: H(nBas,nBas)
    end function qk_Hartree_matrix_AO_basis

    integer(c_int) function qk_exchange_matrix_AO_basis(ctx, nBas, P, ERI, K) &
        bind(C, name="qk_exchange_matrix_AO_basis")
      import c_int, c_ptr, c_double
      type(c_ptr), value            :: ctx
      integer(c_int), value         :: nBas
      real(c_double), intent(in)    :: P(nBas,nBas), ERI(nBas,nBas,nBas,nBas)
      real(c_double), intent(out)   :: K(nBas,nBas)
    end function qk_exchange_matrix_AO_basis

    integer(c_int) function qk_qsRGW(ctx, prm, nBas, nOrb, nC, nO, nV, nR, nS, eHF, cHF, PHF, S, T, &
        V, Hc, X, ERI_AO, eGW, c, P, SigC, Z, EqsGW, EcRPA, EcGM, nSCF, Conv) bind(C, name="qk_qsRGW")
      import c_int, c_ptr, c_double, qk_gw_params
      type(c_ptr), value            :: ctx
      type(qk_gw_params), intent(in):: prm
      integer(c_int), value         :: nBas, nOrb, nC, nO, nV, nR, nS
      real(c_double), intent(in)    :: eHF(nOrb), cHF(nBas,nOrb), PHF(nBas,nBas)
      real(c_double), intent(in)    :: S(nBas,nBas), T(nBas,nBas), V(nBas,nBas), Hc(nBas,nBas)
      real(c_double), intent(in)    :: X(nBas,nOrb), ERI_AO(nBas,nBas,nBas,nBas)
      real(c_double), intent(out)   :: eGW(nOrb), c(nBas,nOrb), P(nBas,nBas), SigC(nOrb,nOrb)
      real(c_double), intent(out)   :: Z(nOrb), EqsGW, EcRPA, EcGM, Conv
      integer(c_int), intent(out)   :: nSCF
    end function qk_qsRGW

    ! QKD_* bits recorded on the device during the context's last call (warnings such as a
    ! negative A-B eigenvalue or a Newton search that used all maxIt steps)
    integer(c_int) function qk_last_device_status(ctx) bind(C, name="qk_last_device_status")
      import c_int, c_ptr
      type(c_ptr), value            :: ctx
    end function qk_last_device_status

  end interface

end module qk_gw_module
