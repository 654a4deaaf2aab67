!==========================================================================
! BSAMGpuHost: the calls the BSAM 1.2 Fortran host makes into libbsamg,
! written against the reference's own modules (NodeInfoDef, TreeOps,
! ProblemDef).  They replace, unchanged in meaning:
!
! * the body of MultigridIterations (LIBRARY/afasroutines.f90:48-110): one
!   bsamg_multigrid_iterations call, then the reference's per-V-cycle print;
! * the CopyQToQold loop of TakeTimeSteps (LIBRARY/bsamroutines.f90:
!   700-702);
! * after each regrid (TakeTimeSteps, bsamroutines.f90:682-702, once AMR
!   and the deletion of the old mesh are done) the mesh moves to the device:
!   GpuUploadMesh walks the levels minlevel..finestlevel with ApplyOnLevel
!   (treeops.f90:515-552, the reference's visiting order), adds every node
!   with its parent, commits, and uploads q and qold.  Node ids are written
!   into info%ngrid (a label the reference only prints; ReadQ sets it to
!   -13, bsaminputoutput.f90:370), so a child finds its parent's id through
!   GetParentInfo (treeops.f90:889-898);
! * before anything on the host reads info%q (WriteQ, AfterStepStatistics
!   on the host, the next regrid), GpuDownloadQ brings q back.
!
! The problem plugin is chosen by name (bsamg_problem_kind): 'ch' for
! PROBLEM/CH (params dt, eps), 'biogrowth' for PROBLEM/BioGrowth (dt, eps,
! gamma, lambda, czero).  Every non-zero status stops the run (BSAMGCheck).
!==========================================================================
MODULE BSAMGpuHost
USE ISO_C_BINDING
USE BSAMGpu
USE NodeInfoDef
IMPLICIT NONE
PRIVATE
PUBLIC:: GpuInit, GpuFinalize, GpuUploadMesh, GpuDownloadQ, GpuCopyQToQold, MultigridIterationsGpu
!
TYPE(C_PTR), SAVE:: gpuctx = C_NULL_PTR, gpuhier = C_NULL_PTR
INTEGER(C_INT), SAVE:: gpukind = 0, gpumode = BSAMG_MODE_FP64
REAL(C_DOUBLE), DIMENSION(1:8), SAVE:: gpuparams
INTEGER(C_INT), SAVE:: gpunparams = 0, nextid = 0
!
CONTAINS
!
! Once, after SetProb: the device, the plugin by name, its parameters (dt
! first, then the problem's own, as problemdata.dat gives them) and the
! mode (BSAMG_MODE_FP64, the drop-in, or BSAMG_MODE_MIXED).
SUBROUTINE GpuInit(device, problem, params, mode)
INTEGER, INTENT(IN):: device, mode
CHARACTER(LEN=*), INTENT(IN):: problem
REAL(KIND=r8), DIMENSION(:), INTENT(IN):: params
CALL BSAMGCheck(bsamg_init(INT(device, C_INT), 0_C_SIZE_T, gpuctx), 'bsamg_init')
CALL BSAMGCheck(bsamg_problem_kind(TRIM(problem)//C_NULL_CHAR, gpukind), 'bsamg_problem_kind')
gpunparams = SIZE(params)
gpuparams(1:gpunparams) = params
gpumode = INT(mode, C_INT)
END SUBROUTINE GpuInit
!
SUBROUTINE GpuFinalize
IF(C_ASSOCIATED(gpuhier)) CALL BSAMGCheck(bsamg_hier_destroy(gpuhier), 'bsamg_hier_destroy')
CALL BSAMGCheck(bsamg_finalize(gpuctx), 'bsamg_finalize')
gpuhier = C_NULL_PTR; gpuctx = C_NULL_PTR
END SUBROUTINE GpuFinalize
!
! After the regrid: a new device hierarchy for the current mesh.
SUBROUTINE GpuUploadMesh
USE TreeOps, ONLY: ApplyOnLevel
TYPE(funcparam):: dummy
INTEGER:: level
IF(C_ASSOCIATED(gpuhier)) CALL BSAMGCheck(bsamg_hier_destroy(gpuhier), 'bsamg_hier_destroy')
gpuparams(1) = dt
CALL BSAMGCheck(bsamg_hier_create(gpuctx, INT(ndims, C_INT), INT(nrvarsof(), C_INT), INT(mbcof(), C_INT), &
                gpukind, gpuparams, gpunparams, qpo, gpuhier), 'bsamg_hier_create')
nextid = 0
DO level = minlevel, finestlevel
  CALL ApplyOnLevel(level, AddNodeToGpu, dummy)
END DO
CALL BSAMGCheck(bsamg_commit(gpuhier), 'bsamg_commit')
DO level = minlevel, finestlevel
  CALL ApplyOnLevel(level, PutNodeFields, dummy)
END DO
END SUBROUTINE GpuUploadMesh
!
! info%q of every node back from the device.
SUBROUTINE GpuDownloadQ
USE TreeOps, ONLY: ApplyOnLevel
TYPE(funcparam):: dummy
INTEGER:: level
DO level = minlevel, finestlevel
  CALL ApplyOnLevel(level, GetNodeQ, dummy)
END DO
END SUBROUTINE GpuDownloadQ
!
! The CopyQToQold loop of TakeTimeSteps (bsamroutines.f90:700-702).
SUBROUTINE GpuCopyQToQold
CALL BSAMGCheck(bsamg_copy_q_to_qold(gpuhier, INT(minlevel, C_INT), INT(finestlevel, C_INT)), &
                'bsamg_copy_q_to_qold')
END SUBROUTINE GpuCopyQToQold
!
! The body of MultigridIterations (afasroutines.f90:48-110): FillDown,
! sources, then V-cycles until ErrorAFAS(finestlevel) < qerrortol or
! maxvcycles, all on the device; the per-V-cycle print is kept.
SUBROUTINE MultigridIterationsGpu
INTEGER(C_INT):: ncycles
INTEGER:: itmg
REAL(C_DOUBLE), DIMENSION(1:maxvcycles):: residuals
CALL BSAMGCheck(bsamg_multigrid_iterations(gpuhier, INT(finestlevel, C_INT), INT(minlevel, C_INT), &
                INT(nsmoothingpasses, C_INT), INT(maxvcycles, C_INT), REAL(qerrortol, C_DOUBLE), &
                INT(updateauxfreq, C_INT), INT(errortype, C_INT), gpumode, 0_C_INT, ncycles, residuals), &
                'MultigridIterations')
DO itmg = 1, ncycles
  PRINT *, 'it =', itmg, ' residual =', residuals(itmg)
END DO
END SUBROUTINE MultigridIterationsGpu
!
! ---- ApplyOnLevel callbacks ----
!
INTEGER FUNCTION AddNodeToGpu(info, dummy)
USE TreeOps, ONLY: GetParentInfo, err_OK
TYPE(nodeinfo):: info
TYPE(funcparam):: dummy
TYPE(nodeinfo), POINTER:: parent
INTEGER(C_INT):: pid
INTEGER(C_INT), DIMENSION(1:3):: mx
INTEGER(C_INT), DIMENSION(1:6):: mglobal, mbounds, mthbc
REAL(C_DOUBLE), DIMENSION(1:3):: dx, xlower
AddNodeToGpu = err_OK
IF(info%tobedeleted .OR. (.NOT. info%activegrid)) RETURN
nextid = nextid+1
info%ngrid = nextid
pid = -1
IF(info%level>minlevel) THEN
  IF(GetParentInfo(parent)/=err_OK) THEN
    PRINT *, 'BSAM 1.2 GPU error: a node above minlevel has no parent'
    STOP
  END IF
  pid = INT(parent%ngrid, C_INT)
END IF
mx = 1; mglobal = 1; mbounds = 1; dx = 0.0_r8; xlower = 0.0_r8
mx(1:ndims) = info%mx(1:ndims)
mglobal(1:2*ndims-1:2) = info%mglobal(1:ndims,1); mglobal(2:2*ndims:2) = info%mglobal(1:ndims,2)
mbounds(1:2*ndims-1:2) = info%mbounds(1:ndims,1); mbounds(2:2*ndims:2) = info%mbounds(1:ndims,2)
mthbc(1:6) = info%mthbc(1:6)
dx(1:ndims) = info%dx(1:ndims); xlower(1:ndims) = info%xlower(1:ndims)
CALL BSAMGCheck(bsamg_patch_add(gpuhier, INT(info%level, C_INT), INT(info%ngrid, C_INT), pid, mx, mglobal, &
                mbounds, mthbc, dx, xlower), 'bsamg_patch_add')
END FUNCTION AddNodeToGpu
!
INTEGER FUNCTION PutNodeFields(info, dummy)
USE TreeOps, ONLY: err_OK
TYPE(nodeinfo):: info
TYPE(funcparam):: dummy
PutNodeFields = err_OK
IF(info%tobedeleted .OR. (.NOT. info%activegrid)) RETURN
CALL BSAMGCheck(bsamg_put_field(gpuhier, INT(info%ngrid, C_INT), BSAMG_FIELD_Q, info%q, &
                INT(SIZE(info%q), C_SIZE_T)), 'bsamg_put_field(q)')
CALL BSAMGCheck(bsamg_put_field(gpuhier, INT(info%ngrid, C_INT), BSAMG_FIELD_QOLD, info%qold, &
                INT(SIZE(info%qold), C_SIZE_T)), 'bsamg_put_field(qold)')
END FUNCTION PutNodeFields
!
INTEGER FUNCTION GetNodeQ(info, dummy)
USE TreeOps, ONLY: err_OK
TYPE(nodeinfo):: info
TYPE(funcparam):: dummy
GetNodeQ = err_OK
IF(info%tobedeleted .OR. (.NOT. info%activegrid)) RETURN
CALL BSAMGCheck(bsamg_get_field(gpuhier, INT(info%ngrid, C_INT), BSAMG_FIELD_Q, info%q, &
                INT(SIZE(info%q), C_SIZE_T)), 'bsamg_get_field(q)')
END FUNCTION GetNodeQ
!
! nrvars and mbc of the run, from the root node
INTEGER FUNCTION nrvarsof()
USE TreeOps, ONLY: GetRootInfo
TYPE(nodeinfo), POINTER:: root
INTEGER:: ierr
ierr = GetRootInfo(root)
nrvarsof = root%nrvars
END FUNCTION nrvarsof
!
INTEGER FUNCTION mbcof()
USE TreeOps, ONLY: GetRootInfo
TYPE(nodeinfo), POINTER:: root
INTEGER:: ierr
ierr = GetRootInfo(root)
mbcof = root%mbc
END FUNCTION mbcof
!
END MODULE BSAMGpuHost
