! ermod_gpu.f90 -- ISO_C_BINDING interface to libermod_gb300.so (include/ermod_gpu.h).
!
! A Fortran ERmod host keeps enganal/setconf/insertion/engstore and replaces the body of
! engconst (engproc.F90:355-392) by calls to these routines.  Arrays are passed exactly
! as engmain.F90 holds them: column-major, 1-based index values, charges already scaled
! by 18.22261721, temperature as kT in kcal/mol.
module ermod_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: ERMOD_ABI_VERSION = 2
  integer(c_int), parameter :: ERMOD_OK = 0, ERMOD_E_ENG_MIN = 101, ERMOD_E_ENG_SFT = 102, &
       ERMOD_E_ENG_BUG = 103, ERMOD_E_ENG_CNS = 104, ERMOD_E_RCP_CNS = 105, ERMOD_E_RCP_FST = 106, &
       ERMOD_E_INS_GEO = 107, ERMOD_E_SET_PRS = 108, ERMOD_E_ENG_SLB = 109, ERMOD_W_MBIN = 110, &
       ERMOD_E_INS_SIZ = 111
  integer(c_int), parameter :: ERMOD_PRECISION_FP64 = 0, ERMOD_PRECISION_MIXED = 1

  type, bind(C) :: ermod_params
     integer(c_int32_t) :: abi_version, slttype, estype, cltype, ljswitch, splodr
     integer(c_int32_t) :: ms1max, ms2max, ms3max, wgtslf, corrcal, selfcal
     integer(c_int32_t) :: force_calculation, precision, batch, count_mirror
     real(c_double) :: elecut, lwljcut, upljcut, screen, temp, block_threshold
     integer(c_int32_t) :: boxshp, finish_group
  end type ermod_params

  interface
     subroutine ermod_default_params(p) bind(C, name="ermod_default_params")
       import :: ermod_params
       type(ermod_params), intent(out) :: p
     end subroutine
     integer(c_int) function ermod_create(p, device, ctx) bind(C, name="ermod_create")
       import :: ermod_params, c_int, c_ptr
       type(ermod_params), intent(in) :: p
       integer(c_int), value :: device
       type(c_ptr), intent(out) :: ctx
     end function
     integer(c_int) function ermod_destroy(ctx) bind(C, name="ermod_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function ermod_set_topology(ctx, nummol, numatm, mol_begin_index, sluvid, uvspec, &
          charge, ljtype, ljtype_max, ljene_mat, ljlensq_mat) bind(C, name="ermod_set_topology")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: nummol, numatm, ljtype_max
       integer(c_int), intent(in) :: mol_begin_index(*), sluvid(*), uvspec(*), ljtype(*)
       real(c_double), intent(in) :: charge(*), ljene_mat(*), ljlensq_mat(*)
     end function
     integer(c_int) function ermod_set_bins(ctx, numslv, uvmax, uvsoft, uvcrd, esmax, escrd) &
          bind(C, name="ermod_set_bins")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: numslv, esmax
       integer(c_int), intent(in) :: uvmax(*), uvsoft(*)
       real(c_double), intent(in) :: uvcrd(*), escrd(*)
     end function
     integer(c_int) function ermod_set_aggregate(ctx, host_mol, sitemass) bind(C, name="ermod_set_aggregate")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), intent(in) :: host_mol(*)
       real(c_double), intent(in) :: sitemass(*)
     end function
     integer(c_int) function ermod_set_reference_structure(ctx, ref_mol, refhost_crd, refhost_weight, &
          refslt_natom, refslt_crd, refslt_weight) bind(C, name="ermod_set_reference_structure")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), intent(in) :: ref_mol(*)
       real(c_double), intent(in) :: refhost_crd(*), refhost_weight(*), refslt_crd(*), refslt_weight(*)
       integer(c_int), value :: refslt_natom
     end function
     ! flexible solute (slttype 3): SltConf's structures conf(3, nsite, nconf), SltWght's
     ! weights (nweight 0: none), getsolute's insstructure window
     integer(c_int) function ermod_set_solute_library(ctx, nconf, nsite, conf, nweight, weight, &
          insstructure, lwstr, upstr) bind(C, name="ermod_set_solute_library")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: nconf, nsite, nweight, insstructure
       real(c_double), intent(in) :: conf(*), weight(*)
       real(c_double), value :: lwstr, upstr
     end function
     integer(c_int) function ermod_set_configuration_check(ctx, insposition, lwreg, upreg, insstructure, &
          lwstr, upstr) bind(C, name="ermod_set_configuration_check")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: insposition, insstructure
       real(c_double), value :: lwreg, upreg, lwstr, upstr
     end function
     integer(c_int) function ermod_frame(ctx, sitepos, cell, stat_weight_system) bind(C, name="ermod_frame")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: sitepos(*), cell(*)
       real(c_double), value :: stat_weight_system
     end function
     integer(c_int) function ermod_placements(ctx, nplace, tagslt, solute_sitepos, stat_weight_solute, &
          uvengy_out, flceng_out) bind(C, name="ermod_placements")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: nplace
       integer(c_int), intent(in) :: tagslt(*)
       type(c_ptr), value :: solute_sitepos, stat_weight_solute, uvengy_out, flceng_out
     end function
     integer(c_int) function ermod_clear(ctx) bind(C, name="ermod_clear")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function ermod_get_accum(ctx, edens, ecorr, eself, slnuv, minuv, maxuv, scalars, &
          ecorr_count) bind(C, name="ermod_get_accum")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, edens, ecorr, eself, slnuv, minuv, maxuv, scalars, ecorr_count
     end function
     integer(c_int) function ermod_error_info(ctx, placement, molecule, energy) bind(C, name="ermod_error_info")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: placement, molecule
       real(c_double), intent(out) :: energy
     end function
     integer(c_int) function ermod_adjoint_enable(ctx, solute_mol, cmbrule) bind(C, name="ermod_adjoint_enable")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: solute_mol, cmbrule
     end function
     integer(c_int) function ermod_adjoint_get(ctx, grad, weight, nparam) bind(C, name="ermod_adjoint_get")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: grad(*), weight(*)   ! grad(ermax, 3*nsite) in Fortran order
       integer(c_int), intent(out) :: nparam
     end function
  end interface
end module ermod_gpu
