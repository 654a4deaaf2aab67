!==========================================================================
! BSAMGpu: ISO_C_BINDING interface of libbsamg (include/bsamg.h) for the
! BSAM 1.2 Fortran 95 host.  One interface per C entry point, with the C
! argument kinds (VALUE for scalars passed by value, by reference for
! pointers and arrays), the status codes and the field, mode and problem
! constants.  BSAMGCheck turns a non-zero status into the reference's
! PRINT + STOP convention (e.g. LIBRARY/bsamstorage.f90:93-96).
!
! Build: add this file before afasroutines.f90 in the makefile's object
! list (PROBLEM/CH/makefile:22-24) and link libbsamg.so.
!==========================================================================
MODULE BSAMGpu
USE ISO_C_BINDING
IMPLICIT NONE
!
! status codes
INTEGER(C_INT), PARAMETER:: BSAMG_OK = 0, BSAMG_ERR_ARG = -1, BSAMG_ERR_CUDA = -2, &
                            BSAMG_ERR_BUDGET = -3, BSAMG_ERR_NOT_CONVERGED = -4, &
                            BSAMG_ERR_NONFINITE = -5, BSAMG_ERR_UNSUPPORTED = -6, &
                            BSAMG_ERR_NOT_FOUND = -7, BSAMG_ERR_IO = -8
! problem plugins shipped with the library (others: bsamg_problem_kind)
INTEGER(C_INT), PARAMETER:: BSAMG_PROBLEM_CH = 1, BSAMG_PROBLEM_BIOGROWTH = 2, &
                            BSAMG_PROBLEM_GROWTH = 3
! fields of a node (nodeinfodef.f90:184-214)
INTEGER(C_INT), PARAMETER:: BSAMG_FIELD_Q = 0, BSAMG_FIELD_QOLD = 1, BSAMG_FIELD_QC = 2, &
                            BSAMG_FIELD_F = 3, BSAMG_FIELD_RF = 4, BSAMG_FIELD_FTMP = 5
INTEGER(C_INT), PARAMETER:: BSAMG_MODE_FP64 = 0, BSAMG_MODE_MIXED = 1
INTEGER(C_INT), PARAMETER:: BSAMG_TAG_CH = 0, BSAMG_TAG_GRADIENT = 1
INTEGER(C_INT), PARAMETER:: BSAMG_NOALLOC_MAX_CELLS = 16777216
!
! regrid parameters (griddata.dat's per-level arrays, indices 0:10)
TYPE, BIND(C):: bsamg_regrid_params
  INTEGER(C_INT):: maxlevel, tagging, initial, maxside, first_id
  INTEGER(C_INT):: ibuffer(0:10), minimumgridpoints(0:10)
  REAL(C_DOUBLE):: qtolerance(0:10), desiredfillratio(0:10)
END TYPE bsamg_regrid_params
!
INTERFACE
  FUNCTION bsamg_problem_kind(name, kind) BIND(C, NAME='bsamg_problem_kind') RESULT(status)
    IMPORT
    CHARACTER(KIND=C_CHAR):: name(*)
    INTEGER(C_INT):: kind
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_problem_info(kind, nrvars, nparams, has_mixed) BIND(C, NAME='bsamg_problem_info') RESULT(status)
    IMPORT
    INTEGER(C_INT), VALUE:: kind
    INTEGER(C_INT):: nrvars, nparams, has_mixed
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_init(device, hbm_budget_bytes, ctx) BIND(C, NAME='bsamg_init') RESULT(status)
    IMPORT
    INTEGER(C_INT), VALUE:: device
    INTEGER(C_SIZE_T), VALUE:: hbm_budget_bytes
    TYPE(C_PTR):: ctx
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_finalize(ctx) BIND(C, NAME='bsamg_finalize') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_ctx_usage(ctx, used, budget) BIND(C, NAME='bsamg_ctx_usage') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    INTEGER(C_SIZE_T):: used, budget
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_ctx_set_blocking_wait(ctx, on) BIND(C, NAME='bsamg_ctx_set_blocking_wait') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    INTEGER(C_INT), VALUE:: on
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_hier_create(ctx, ndims, nrvars, mbc, problem_kind, params, nparams, qpo, h) &
      BIND(C, NAME='bsamg_hier_create') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    INTEGER(C_INT), VALUE:: ndims, nrvars, mbc, problem_kind
    REAL(C_DOUBLE):: params(*)
    INTEGER(C_INT), VALUE:: nparams
    REAL(C_DOUBLE):: qpo(*)
    TYPE(C_PTR):: h
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_hier_destroy(h) BIND(C, NAME='bsamg_hier_destroy') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_regrid(h, prm, qinit, user, hnew) BIND(C, NAME='bsamg_regrid') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    TYPE(bsamg_regrid_params):: prm
    TYPE(C_FUNPTR), VALUE:: qinit
    TYPE(C_PTR), VALUE:: user
    TYPE(C_PTR):: hnew
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_patch_add(h, level, id, parent_id, mx, mglobal, mbounds, mthbc, dx, xlower) &
      BIND(C, NAME='bsamg_patch_add') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, id, parent_id
    INTEGER(C_INT):: mx(3), mglobal(6), mbounds(6), mthbc(6)
    REAL(C_DOUBLE):: dx(3), xlower(3)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_build_uniform(h, mx, minlevel, mthbc, xlower, xupper) BIND(C, NAME='bsamg_build_uniform') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: mx(3)
    INTEGER(C_INT), VALUE:: minlevel
    INTEGER(C_INT):: mthbc(6)
    REAL(C_DOUBLE):: xlower(3), xupper(3)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_commit(h) BIND(C, NAME='bsamg_commit') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_num_patches(h, n) BIND(C, NAME='bsamg_num_patches') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_level_range(h, minlevel, maxlevel) BIND(C, NAME='bsamg_level_range') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: minlevel, maxlevel
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_patch_info(h, index, info, dxl) BIND(C, NAME='bsamg_patch_info') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: index
    INTEGER(C_INT):: info(*)
    REAL(C_DOUBLE):: dxl(*)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_field_size(h, id, field) BIND(C, NAME='bsamg_field_size') RESULT(n)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: id, field
    INTEGER(C_SIZE_T):: n
  END FUNCTION
  FUNCTION bsamg_put_field(h, id, field, a, n) BIND(C, NAME='bsamg_put_field') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: id, field
    REAL(C_DOUBLE):: a(*)
    INTEGER(C_SIZE_T), VALUE:: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_get_field(h, id, field, a, n) BIND(C, NAME='bsamg_get_field') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: id, field
    REAL(C_DOUBLE):: a(*)
    INTEGER(C_SIZE_T), VALUE:: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_put_field_section(h, id, field, a, lo, hi) BIND(C, NAME='bsamg_put_field_section') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: id, field
    REAL(C_DOUBLE):: a(*)
    INTEGER(C_INT):: lo(4), hi(4)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_get_field_section(h, id, field, a, lo, hi) BIND(C, NAME='bsamg_get_field_section') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: id, field
    REAL(C_DOUBLE):: a(*)
    INTEGER(C_INT):: lo(4), hi(4)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_relax_level_color(h, level, ipass) BIND(C, NAME='bsamg_relax_level_color') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, ipass
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_set_ghost(h, level, ipass) BIND(C, NAME='bsamg_set_ghost') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, ipass
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_level_relax(h, level, nsmooth) BIND(C, NAME='bsamg_level_relax') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, nsmooth
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_fill_down(h, field, finestlevel, minlevel) BIND(C, NAME='bsamg_fill_down') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: field, finestlevel, minlevel
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_copy_q_to_qold(h, minlevel, finestlevel) BIND(C, NAME='bsamg_copy_q_to_qold') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: minlevel, finestlevel
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_vcycle(h, level, minlevel, nsmooth) BIND(C, NAME='bsamg_vcycle') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, minlevel, nsmooth
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_residual_norm(h, level, errortype, norm) BIND(C, NAME='bsamg_residual_norm') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, errortype
    REAL(C_DOUBLE):: norm
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_multigrid_iterations(h, finestlevel, minlevel, nsmooth, maxvcycles, qerrortol, &
      updateauxfreq, errortype, mode, strict, ncycles, residuals) &
      BIND(C, NAME='bsamg_multigrid_iterations') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: finestlevel, minlevel, nsmooth, maxvcycles
    REAL(C_DOUBLE), VALUE:: qerrortol
    INTEGER(C_INT), VALUE:: updateauxfreq, errortype, mode, strict
    INTEGER(C_INT):: ncycles
    REAL(C_DOUBLE):: residuals(*)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_time_step(h, first, finestlevel, minlevel, nsmooth, maxvcycles, qerrortol, &
      updateauxfreq, errortype, mode, strict, ncycles, residuals) BIND(C, NAME='bsamg_time_step') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: first, finestlevel, minlevel, nsmooth, maxvcycles
    REAL(C_DOUBLE), VALUE:: qerrortol
    INTEGER(C_INT), VALUE:: updateauxfreq, errortype, mode, strict
    INTEGER(C_INT):: ncycles
    REAL(C_DOUBLE):: residuals(*)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_after_step_stats(h, finestlevel, integral, meshsize) BIND(C, NAME='bsamg_after_step_stats') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: finestlevel
    REAL(C_DOUBLE):: integral(2)
    INTEGER(C_LONG_LONG):: meshsize
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_write_q(h, path, time, finestlevel) BIND(C, NAME='bsamg_write_q') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    CHARACTER(KIND=C_CHAR):: path(*)
    REAL(C_DOUBLE), VALUE:: time
    INTEGER(C_INT), VALUE:: finestlevel
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_write_uniform_q(h, path, time, finestlevel) BIND(C, NAME='bsamg_write_uniform_q') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    CHARACTER(KIND=C_CHAR):: path(*)
    REAL(C_DOUBLE), VALUE:: time
    INTEGER(C_INT), VALUE:: finestlevel
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_read_q(root, path, first_id, time, h) BIND(C, NAME='bsamg_read_q') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: root
    CHARACTER(KIND=C_CHAR):: path(*)
    INTEGER(C_INT), VALUE:: first_id
    REAL(C_DOUBLE):: time
    TYPE(C_PTR):: h
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_format_f25_12(x, out) BIND(C, NAME='bsamg_format_f25_12') RESULT(status)
    IMPORT
    REAL(C_DOUBLE), VALUE:: x
    CHARACTER(KIND=C_CHAR):: out(*)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_format_stats_line(time, integral, meshsize, out, n) BIND(C, NAME='bsamg_format_stats_line') &
      RESULT(status)
    IMPORT
    REAL(C_DOUBLE), VALUE:: time
    REAL(C_DOUBLE):: integral(2)
    INTEGER(C_LONG_LONG), VALUE:: meshsize
    CHARACTER(KIND=C_CHAR):: out(*)
    INTEGER(C_SIZE_T), VALUE:: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_seed_spinodal(h, id, seed, mean, amp) BIND(C, NAME='bsamg_seed_spinodal') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: id
    INTEGER(C_LONG_LONG), VALUE:: seed
    REAL(C_DOUBLE), VALUE:: mean, amp
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_sync(h) BIND(C, NAME='bsamg_sync') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_stream(h, stream) BIND(C, NAME='bsamg_stream') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    TYPE(C_PTR):: stream
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_launch_count(h, n) BIND(C, NAME='bsamg_launch_count') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_LONG_LONG):: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_graph_stats(h, instantiated, updated) BIND(C, NAME='bsamg_graph_stats') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: instantiated, updated
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_set_params(h, params, nparams) BIND(C, NAME='bsamg_set_params') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    REAL(C_DOUBLE):: params(*)
    INTEGER(C_INT), VALUE:: nparams
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_hier_reset(h) BIND(C, NAME='bsamg_hier_reset') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_set_box_sweep(h, kind) BIND(C, NAME='bsamg_set_box_sweep') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: kind
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_set_tail_cells(h, cells) BIND(C, NAME='bsamg_set_tail_cells') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_LONG_LONG), VALUE:: cells
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_set_solve(h, mode, ctas, threads, tile, solo_cells) BIND(C, NAME='bsamg_set_solve') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: mode, ctas, threads, tile
    INTEGER(C_LONG_LONG), VALUE:: solo_cells
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_get_solve(h, mode, ctas, threads, tile, solo_cells) BIND(C, NAME='bsamg_get_solve') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT):: mode, ctas, threads, tile
    INTEGER(C_LONG_LONG):: solo_cells
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_solve_info(h, info, n) BIND(C, NAME='bsamg_solve_info') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_LONG_LONG):: info(*)
    INTEGER(C_INT), VALUE:: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_ctx_set_autotune(ctx, on) BIND(C, NAME='bsamg_ctx_set_autotune') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    INTEGER(C_INT), VALUE:: on
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_tune_save(ctx, path) BIND(C, NAME='bsamg_tune_save') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    CHARACTER(KIND=C_CHAR):: path(*)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_tune_load(ctx, path) BIND(C, NAME='bsamg_tune_load') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    CHARACTER(KIND=C_CHAR):: path(*)
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_tune_count(ctx, n) BIND(C, NAME='bsamg_tune_count') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ctx
    INTEGER(C_INT):: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_regrid_timing(h, ms, n) BIND(C, NAME='bsamg_regrid_timing') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    REAL(C_DOUBLE):: ms(*)
    INTEGER(C_INT), VALUE:: n
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_solve_trace(h, enable) BIND(C, NAME='bsamg_solve_trace') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: enable
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_solve_trace_read(h, cap, op, n, cycles, count) BIND(C, NAME='bsamg_solve_trace_read') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: cap
    INTEGER(C_INT):: op(*), n(*)
    INTEGER(C_LONG_LONG):: cycles(*)
    INTEGER(C_INT):: count
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_mark(h, slot) BIND(C, NAME='bsamg_mark') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: slot
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_elapsed_ms(h, a, b, ms) BIND(C, NAME='bsamg_elapsed_ms') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: a, b
    REAL(C_DOUBLE):: ms
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_time_smoother(h, level, mode, reps, ms_per_launch) BIND(C, NAME='bsamg_time_smoother') &
      RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, mode, reps
    REAL(C_DOUBLE):: ms_per_launch
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_smoother_colours(h, level, mode, colours) BIND(C, NAME='bsamg_smoother_colours') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: h
    INTEGER(C_INT), VALUE:: level, mode
    INTEGER(C_INT):: colours
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_ch_residual_norm_noalloc(q, f, ndims, mx, h, dt, eps, errortype, norm_out, stream) &
      BIND(C, NAME='bsamg_ch_residual_norm_noalloc') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: q, f
    INTEGER(C_INT), VALUE:: ndims
    INTEGER(C_INT):: mx(3)
    REAL(C_DOUBLE), VALUE:: h, dt, eps
    INTEGER(C_INT), VALUE:: errortype
    TYPE(C_PTR), VALUE:: norm_out, stream
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_host_register(ptr, bytes) BIND(C, NAME='bsamg_host_register') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ptr
    INTEGER(C_SIZE_T), VALUE:: bytes
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_host_unregister(ptr) BIND(C, NAME='bsamg_host_unregister') RESULT(status)
    IMPORT
    TYPE(C_PTR), VALUE:: ptr
    INTEGER(C_INT):: status
  END FUNCTION
  FUNCTION bsamg_strerror(status) BIND(C, NAME='bsamg_strerror') RESULT(text)
    IMPORT
    INTEGER(C_INT), VALUE:: status
    TYPE(C_PTR):: text
  END FUNCTION
  FUNCTION bsamg_last_error_detail() BIND(C, NAME='bsamg_last_error_detail') RESULT(text)
    IMPORT
    TYPE(C_PTR):: text
  END FUNCTION
END INTERFACE
!
CONTAINS
!
! A non-zero status becomes the reference's error convention: a message and
! STOP (e.g. LIBRARY/bsamstorage.f90:93-96).
SUBROUTINE BSAMGCheck(status, what)
INTEGER(C_INT), INTENT(IN):: status
CHARACTER(LEN=*), INTENT(IN):: what
IF(status/=BSAMG_OK) THEN
  PRINT *, 'BSAM 1.2 GPU error in ', what, ': ', TRIM(CString(bsamg_strerror(status))), &
           ' (', status, ') ', TRIM(CString(bsamg_last_error_detail()))
  STOP
END IF
END SUBROUTINE BSAMGCheck
!
! A C string returned by the library as a Fortran string (at most 256
! characters).
FUNCTION CString(p) RESULT(s)
TYPE(C_PTR), INTENT(IN):: p
CHARACTER(LEN=256):: s
CHARACTER(KIND=C_CHAR), DIMENSION(:), POINTER:: c
INTEGER:: i
s = ' '
IF(.NOT. C_ASSOCIATED(p)) RETURN
CALL C_F_POINTER(p, c, [256])
DO i = 1, 256
  IF(c(i)==C_NULL_CHAR) EXIT
  s(i:i) = c(i)
END DO
END FUNCTION CString
!
END MODULE BSAMGpu
