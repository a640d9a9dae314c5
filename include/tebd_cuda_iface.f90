! tebd_cuda_iface.f90 -- ISO_C_BINDING interfaces of include/tebd_capi.h for a
! Fortran host of OpenTEBD-extended.
! Gammas, Lambdas and labels are passed as C_LOC of the host's own arrays: the
! layouts are the reference's, so nothing is transposed or copied on the host.
MODULE tebd_cuda_iface
USE ISO_C_BINDING
IMPLICIT NONE
TYPE, BIND(C) :: tebd_opts
  INTEGER(C_INT) :: version, device, tot_num, max_filling, svd_mode, max_sweeps, max_batch, reserved
  REAL(C_DOUBLE) :: jacobi_tol
END TYPE tebd_opts
TYPE, BIND(C) :: tebd_stats
  INTEGER(C_LONG_LONG) :: updates, kernel_launches, jacobi_launches, jacobi_sweeps, jacobi_pairs, jacobi_rotations
  REAL(C_DOUBLE) :: jacobi_flops, jacobi_bytes, jacobi_ms, batch_ms
  INTEGER(C_LONG_LONG) :: compact_rows, compact_cols
  REAL(C_DOUBLE) :: qr_flops, qr_ms
  INTEGER(C_LONG_LONG) :: rank_sum
  REAL(C_DOUBLE) :: bidiag_ms
  INTEGER(C_LONG_LONG) :: bidiag_updates
  REAL(C_DOUBLE) :: gebrd_flops, gebrd_ms
  INTEGER(C_LONG_LONG) :: gebrd_launches
  INTEGER(C_LONG_LONG) :: rsvd_updates, rsvd_fallbacks
  REAL(C_DOUBLE) :: rsvd_flops, rsvd_worst_residual
  INTEGER(C_LONG_LONG) :: rsvd_skipped
  REAL(C_DOUBLE) :: tc_ms
  INTEGER(C_LONG_LONG) :: tc_launches
  REAL(C_DOUBLE) :: tc_mma_flops
  INTEGER(C_LONG_LONG) :: rsvd_batches, rsvd_oversample_sum, rsvd_power_sum, rsvd_retries
END TYPE
INTERFACE
  SUBROUTINE tebd_default_opts(o) BIND(C, NAME='tebd_default_opts')
    IMPORT :: tebd_opts
    TYPE(tebd_opts) :: o
  END SUBROUTINE
  INTEGER(C_INT) FUNCTION tebd_create(L, d, chi, mode, o, h) BIND(C, NAME='tebd_create')
    IMPORT :: C_INT, C_PTR, tebd_opts
    INTEGER(C_INT), VALUE :: L, d, chi, mode
    TYPE(tebd_opts) :: o
    TYPE(C_PTR) :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_destroy(h) BIND(C, NAME='tebd_destroy')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_set_gamma(h, site, g) BIND(C, NAME='tebd_set_gamma')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, g
    INTEGER(C_INT), VALUE :: site
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_get_gamma(h, site, g) BIND(C, NAME='tebd_get_gamma')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, g
    INTEGER(C_INT), VALUE :: site
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_set_lambda(h, link, l) BIND(C, NAME='tebd_set_lambda')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, l
    INTEGER(C_INT), VALUE :: link
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_get_lambda(h, link, l) BIND(C, NAME='tebd_get_lambda')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, l
    INTEGER(C_INT), VALUE :: link
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_set_labels(h, link, ll, lr) BIND(C, NAME='tebd_set_labels')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, ll, lr
    INTEGER(C_INT), VALUE :: link
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_get_labels(h, link, ll, lr) BIND(C, NAME='tebd_get_labels')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, ll, lr
    INTEGER(C_INT), VALUE :: link
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_two_site_op(h, link, op2, truncerr) BIND(C, NAME='tebd_two_site_op')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: h, op2
    INTEGER(C_INT), VALUE :: link
    REAL(C_DOUBLE) :: truncerr
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_two_site_op_nc(h, link, op2, truncerr) BIND(C, NAME='tebd_two_site_op_nc')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: h, op2
    INTEGER(C_INT), VALUE :: link
    REAL(C_DOUBLE) :: truncerr
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_trotter_step(h, order, ngates, gates, total) BIND(C, NAME='tebd_trotter_step')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: h, gates
    INTEGER(C_INT), VALUE :: order, ngates
    REAL(C_DOUBLE) :: total
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_one_site_expval(h, op, explist) BIND(C, NAME='tebd_one_site_expval')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, op, explist
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_total_energy(h, nops, hops, energy) BIND(C, NAME='tebd_total_energy')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: h, hops
    INTEGER(C_INT), VALUE :: nops
    REAL(C_DOUBLE) :: energy
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_record_gammas(h, path, kind, append) BIND(C, NAME='tebd_record_gammas')
    IMPORT :: C_INT, C_PTR, C_CHAR
    TYPE(C_PTR), VALUE :: h
    CHARACTER(KIND=C_CHAR) :: path(*)
    CHARACTER(KIND=C_CHAR), VALUE :: kind
    INTEGER(C_INT), VALUE :: append
  END FUNCTION
  ! Swapping / SwappingNC (the handle's mode decides)
  INTEGER(C_INT) FUNCTION tebd_swapping(h, link, truncerr) BIND(C, NAME='tebd_swapping')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: link
    REAL(C_DOUBLE) :: truncerr
  END FUNCTION
  ! TrotterStep with BoundaryCond='P' (order 2 or 5; dense or NC handle)
  INTEGER(C_INT) FUNCTION tebd_trotter_step_pbc(h, order, ngates, gates, total) BIND(C, NAME='tebd_trotter_step_pbc')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: h, gates
    INTEGER(C_INT), VALUE :: order, ngates
    REAL(C_DOUBLE) :: total
  END FUNCTION
  ! intDegFree present: pass C_LOC(Conserv%vi); C_NULL_PTR for the plain form
  INTEGER(C_INT) FUNCTION tebd_set_conserv(h, conserv) BIND(C, NAME='tebd_set_conserv')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, conserv
  END FUNCTION
  ! kept-rank form (no reference counterpart); 0 = the reference's rule
  INTEGER(C_INT) FUNCTION tebd_set_rank_bound(h, bound) BIND(C, NAME='tebd_set_rank_bound')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: h
    REAL(C_DOUBLE), VALUE :: bound
  END FUNCTION
  ! diagnostics, observables, record I/O, canonical forms, allocation-free update
  INTEGER(C_INT) FUNCTION tebd_two_site_op_r(h, link, op2, truncerr) BIND(C, NAME='tebd_two_site_op_r')
    IMPORT :: C_DOUBLE, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: link
    TYPE(C_PTR), VALUE :: op2
    REAL(C_DOUBLE) :: truncerr
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_two_site_op_nc_r(h, link, op2, truncerr) BIND(C, NAME='tebd_two_site_op_nc_r')
    IMPORT :: C_DOUBLE, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: link
    TYPE(C_PTR), VALUE :: op2
    REAL(C_DOUBLE) :: truncerr
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_apply_bonds(h, nbonds, links, gates, truncerr) BIND(C, NAME='tebd_apply_bonds')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: nbonds
    TYPE(C_PTR), VALUE :: links, gates, truncerr
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_canonical_form(h, link) BIND(C, NAME='tebd_canonical_form')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: link
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_canonical_form_all(h) BIND(C, NAME='tebd_canonical_form_all')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_canonical_form_all_nc(h) BIND(C, NAME='tebd_canonical_form_all_nc')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_get_singular_values(h, link, sigma, count) BIND(C, NAME='tebd_get_singular_values')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: link
    TYPE(C_PTR), VALUE :: sigma
    INTEGER(C_INT) :: count
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_get_sweeps(h, link, sweeps) BIND(C, NAME='tebd_get_sweeps')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: link
    INTEGER(C_INT) :: sweeps
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_sync(h) BIND(C, NAME='tebd_sync')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  TYPE(C_PTR) FUNCTION tebd_last_error(h) BIND(C, NAME='tebd_last_error')
    IMPORT :: C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_LONG_LONG) FUNCTION tebd_kernel_launches(h) BIND(C, NAME='tebd_kernel_launches')
    IMPORT :: C_LONG_LONG, C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_set_profiling(h, on) BIND(C, NAME='tebd_set_profiling')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: on
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_get_stats(h, stats) BIND(C, NAME='tebd_get_stats')
    IMPORT :: C_INT, C_PTR, tebd_stats
    TYPE(C_PTR), VALUE :: h
    TYPE(tebd_stats) :: stats
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_reset_stats(h) BIND(C, NAME='tebd_reset_stats')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_measure_fp64_peak(device, tflops) BIND(C, NAME='tebd_measure_fp64_peak')
    IMPORT :: C_DOUBLE, C_INT
    INTEGER(C_INT), VALUE :: device
    REAL(C_DOUBLE) :: tflops
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_autotune(h, nbonds, links, gates, base_ms, best_ms) BIND(C, NAME='tebd_autotune')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: nbonds
    TYPE(C_PTR), VALUE :: links, gates, base_ms, best_ms
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_get_tuning(device, entries, max_entries, count) BIND(C, NAME='tebd_get_tuning')
    IMPORT :: C_INT
    INTEGER(C_INT), VALUE :: device, max_entries
    INTEGER(C_INT) :: entries(10, *)
    INTEGER(C_INT) :: count
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_clear_tuning(device) BIND(C, NAME='tebd_clear_tuning')
    IMPORT :: C_INT
    INTEGER(C_INT), VALUE :: device
  END FUNCTION
  TYPE(C_PTR) FUNCTION tebd_get_stream(h) BIND(C, NAME='tebd_get_stream')
    IMPORT :: C_PTR
    TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_single_site_rho(h, rho) BIND(C, NAME='tebd_single_site_rho')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    TYPE(C_PTR), VALUE :: rho
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_one_site_expval_r(h, op, explist) BIND(C, NAME='tebd_one_site_expval_r')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    TYPE(C_PTR), VALUE :: op, explist
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_two_site_rho(h, link, rho2) BIND(C, NAME='tebd_two_site_rho')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: link
    TYPE(C_PTR), VALUE :: rho2
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_local_energy(h, nops, hops, energy) BIND(C, NAME='tebd_local_energy')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: nops
    TYPE(C_PTR), VALUE :: hops, energy
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_inner_product(hl, hr, val) BIND(C, NAME='tebd_inner_product')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: hl, hr
    TYPE(C_PTR), VALUE :: val  ! <left|right>: two doubles (re, im)
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_chain_entropy(h, entropy) BIND(C, NAME='tebd_chain_entropy')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    TYPE(C_PTR), VALUE :: entropy
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_record_lambdas(h, path, kind, append) BIND(C, NAME='tebd_record_lambdas')
    IMPORT :: C_CHAR, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    CHARACTER(KIND=C_CHAR) :: path(*)
    CHARACTER(KIND=C_CHAR), VALUE :: kind
    INTEGER(C_INT), VALUE :: append
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_record_labels(h, path_left, path_right) BIND(C, NAME='tebd_record_labels')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    TYPE(C_PTR), VALUE :: path_left, path_right
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_read_gamma_lambda(h, lambda_path, gamma_path, kind, chi_now) BIND(C, NAME='tebd_read_gamma_lambda')
    IMPORT :: C_CHAR, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    CHARACTER(KIND=C_CHAR) :: lambda_path(*)
    CHARACTER(KIND=C_CHAR) :: gamma_path(*)
    CHARACTER(KIND=C_CHAR), VALUE :: kind
    INTEGER(C_INT), VALUE :: chi_now
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_read_gamma_lambda_labels(h, lambda_path, gamma_path, left_path, right_path, kind, chi_now) &
      BIND(C, NAME='tebd_read_gamma_lambda_labels')
    IMPORT :: C_CHAR, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    CHARACTER(KIND=C_CHAR) :: lambda_path(*)
    CHARACTER(KIND=C_CHAR) :: gamma_path(*)
    CHARACTER(KIND=C_CHAR) :: left_path(*)
    CHARACTER(KIND=C_CHAR) :: right_path(*)
    CHARACTER(KIND=C_CHAR), VALUE :: kind
    INTEGER(C_INT), VALUE :: chi_now
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_two_site_op_noalloc(L, d, chi, link, gammas, lambdas, op2, truncerr, stream) &
      BIND(C, NAME='tebd_two_site_op_noalloc')
    IMPORT :: C_DOUBLE, C_INT, C_PTR
    INTEGER(C_INT), VALUE :: L, d, chi, link
    TYPE(C_PTR), VALUE :: gammas, lambdas, op2, stream
    REAL(C_DOUBLE) :: truncerr
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_zgemm_tc(nprob, m, n, k, A, stride_a, lda, B, stride_b, ldb, C, stride_c, &
      ldc, form, stream) BIND(C, NAME='tebd_zgemm_tc')
    IMPORT :: C_INT, C_LONG_LONG, C_PTR
    INTEGER(C_INT), VALUE :: nprob, m, n, k, lda, ldb, ldc, form
    INTEGER(C_LONG_LONG), VALUE :: stride_a, stride_b, stride_c
    TYPE(C_PTR), VALUE :: A, B, C, stream
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_set_theta_form(h, form) BIND(C, NAME='tebd_set_theta_form')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: form
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_set_rsvd(h, oversample, power_iters, tol, slices) BIND(C, NAME='tebd_set_rsvd')
    IMPORT :: C_DOUBLE, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h
    INTEGER(C_INT), VALUE :: oversample, power_iters, slices
    REAL(C_DOUBLE), VALUE :: tol
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_create(device, seed, m) BIND(C, NAME='tebd_mlp_create')
    IMPORT :: C_INT, C_LONG_LONG, C_PTR
    INTEGER(C_INT), VALUE :: device
    INTEGER(C_LONG_LONG), VALUE :: seed
    TYPE(C_PTR) :: m
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_destroy(m) BIND(C, NAME='tebd_mlp_destroy')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: m
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_param_count() BIND(C, NAME='tebd_mlp_param_count')
    IMPORT :: C_INT
  END FUNCTION
  TYPE(C_PTR) FUNCTION tebd_mlp_last_error(m) BIND(C, NAME='tebd_mlp_last_error')
    IMPORT :: C_PTR
    TYPE(C_PTR), VALUE :: m
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_get_params(m, params) BIND(C, NAME='tebd_mlp_get_params')
    IMPORT :: C_FLOAT, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: m
    REAL(C_FLOAT) :: params(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_set_params(m, params) BIND(C, NAME='tebd_mlp_set_params')
    IMPORT :: C_FLOAT, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: m
    REAL(C_FLOAT) :: params(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_forward(m, n, x, y) BIND(C, NAME='tebd_mlp_forward')
    IMPORT :: C_FLOAT, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: m
    INTEGER(C_INT), VALUE :: n
    REAL(C_FLOAT) :: x(*), y(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_loss_grad(m, n, x, t, loss, grad) BIND(C, NAME='tebd_mlp_loss_grad')
    IMPORT :: C_DOUBLE, C_FLOAT, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: m
    INTEGER(C_INT), VALUE :: n
    REAL(C_FLOAT) :: x(*), t(*), grad(*)
    REAL(C_DOUBLE) :: loss
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_mlp_train(m, n, x, t, epochs, batch, lr, loss) BIND(C, NAME='tebd_mlp_train')
    IMPORT :: C_DOUBLE, C_FLOAT, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: m
    INTEGER(C_INT), VALUE :: n, epochs, batch
    REAL(C_FLOAT) :: x(*), t(*)
    REAL(C_FLOAT), VALUE :: lr
    REAL(C_DOUBLE) :: loss
  END FUNCTION
  INTEGER(C_INT) FUNCTION tebd_set_rsvd_model(h, m, target) BIND(C, NAME='tebd_set_rsvd_model')
    IMPORT :: C_DOUBLE, C_INT, C_PTR
    TYPE(C_PTR), VALUE :: h, m
    REAL(C_DOUBLE), VALUE :: target
  END FUNCTION
END INTERFACE
END MODULE tebd_cuda_iface
