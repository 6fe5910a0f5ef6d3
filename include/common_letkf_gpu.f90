!=======================================================================
! common_letkf_gpu -- Fortran binding of libletkf_gpu.so (include/letkf_gpu.h)
!
! Drop-in for MODULE common_letkf (common/common_letkf.f90:1-245): a model
! driver replaces "USE common_letkf" by "USE common_letkf_gpu" and links
! -lletkf_gpu.  SUBROUTINE letkf_core keeps the reference's argument list,
! intents and optional arguments; the analysis runs on the GPU in FP64.
! Where the reference STOPs in mtx_eigen (common/common_mtx.f90:61-64,75-78)
! this STOPs too, after printing the library status.
!
! No Fortran compiler exists in the build image, so this file is shipped as
! source; the C entry point it binds is tested from ctypes.
!=======================================================================
MODULE common_letkf_gpu
  USE ISO_C_BINDING
  IMPLICIT NONE
  PRIVATE
  PUBLIC :: letkf_core, nbv

  INTEGER,PARAMETER :: nbv=20    ! common/common_letkf.f90:28

  INTERFACE
    INTEGER(C_INT) FUNCTION letkf_core_c(ne,nobs,nobsl,hdxb,rdiag,rloc,dep,parm_infl, &
                                         trans,transm,pao,rdiag_wloc,minfl) BIND(C,NAME='letkf_core_c')
      IMPORT :: C_INT, C_DOUBLE, C_PTR
      INTEGER(C_INT),VALUE :: ne, nobs, nobsl
      REAL(C_DOUBLE),INTENT(IN) :: hdxb(*), rdiag(*), rloc(*), dep(*)
      REAL(C_DOUBLE),INTENT(INOUT) :: parm_infl
      REAL(C_DOUBLE),INTENT(OUT) :: trans(*)
      TYPE(C_PTR),VALUE :: transm, pao
      INTEGER(C_INT),VALUE :: rdiag_wloc
      REAL(C_DOUBLE),VALUE :: minfl
    END FUNCTION letkf_core_c
    FUNCTION letkf_status_string(st) BIND(C,NAME='letkf_status_string')
      IMPORT :: C_INT, C_PTR
      INTEGER(C_INT),VALUE :: st
      TYPE(C_PTR) :: letkf_status_string
    END FUNCTION letkf_status_string
  END INTERFACE

CONTAINS

SUBROUTINE letkf_core(ne,nobs,nobsl,hdxb,rdiag,rloc,dep,parm_infl,trans,transm,pao,rdiag_wloc,minfl)
  IMPLICIT NONE
  INTEGER,INTENT(IN) :: ne
  INTEGER,INTENT(IN) :: nobs
  INTEGER,INTENT(IN) :: nobsl
  REAL(C_DOUBLE),INTENT(IN) :: hdxb(1:nobs,1:ne)
  REAL(C_DOUBLE),INTENT(IN) :: rdiag(1:nobs)
  REAL(C_DOUBLE),INTENT(IN) :: rloc(1:nobs)
  REAL(C_DOUBLE),INTENT(IN) :: dep(1:nobs)
  REAL(C_DOUBLE),INTENT(INOUT) :: parm_infl
  REAL(C_DOUBLE),INTENT(OUT) :: trans(ne,ne)
  REAL(C_DOUBLE),INTENT(OUT),OPTIONAL,TARGET :: transm(ne)
  REAL(C_DOUBLE),INTENT(OUT),OPTIONAL,TARGET :: pao(ne,ne)
  LOGICAL,INTENT(IN),OPTIONAL :: rdiag_wloc
  REAL(C_DOUBLE),INTENT(IN),OPTIONAL :: minfl
  TYPE(C_PTR) :: p_transm, p_pao
  INTEGER(C_INT) :: wloc, st
  REAL(C_DOUBLE) :: mf

  p_transm = C_NULL_PTR
  p_pao = C_NULL_PTR
  IF (PRESENT(transm)) p_transm = C_LOC(transm)
  IF (PRESENT(pao)) p_pao = C_LOC(pao)
  wloc = 0
  IF (PRESENT(rdiag_wloc)) THEN
    IF (rdiag_wloc) wloc = 1
  END IF
  mf = 0.0d0                      ! <= 0 means absent, as the reference only acts on minfl > 0
  IF (PRESENT(minfl)) mf = minfl
  st = letkf_core_c(INT(ne,C_INT),INT(nobs,C_INT),INT(nobsl,C_INT),hdxb,rdiag,rloc,dep, &
                    parm_infl,trans,p_transm,p_pao,wloc,mf)
  IF (st /= 0) THEN
    WRITE(6,'(A,I4)') '!!! ERROR (letkf_core on GPU): letkf status ',st
    IF (st == 2) STOP 2         ! common/common_mtx.f90:61-64,75-78
    STOP 99
  END IF
END SUBROUTINE letkf_core

END MODULE common_letkf_gpu
