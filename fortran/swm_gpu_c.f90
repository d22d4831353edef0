! swm_gpu_c.f90 -- iso_c_binding interfaces of every entry point of the GB300
! hot path's C-ABI (include/swm_gpu.h), for the reference's Fortran host code
! (vvshashkin/cubedsphere_sbp_swm).  One interface per C function, same name,
! same argument order:
!   handles (swm_ctx*, swm_state*, ...)  -> type(c_ptr), value
!   handle outputs (swm_ctx** ...)        -> type(c_ptr), intent(out)
!   host arrays (const double* ...)       -> real(c_double) :: a(*)
!   arrays that may be NULL               -> type(c_ptr), value (c_loc or c_null_ptr)
!   strings (const char*)                 -> character(kind=c_char) :: s(*),
!                                            passed as trim(name)//c_null_char
! Every function returns SWM_OK (0) or a negative SWM_E_* code; the message
! of the last failure is swm_last_error (swm_error_message converts it).
! Host arrays are the reference's tile arrays of one tile per panel, FP64,
! (N+1) x (N+1) per panel, i fastest, the six panels one after another.
module swm_gpu_c
use iso_c_binding
implicit none

integer(c_int), parameter :: SWM_OK = 0, SWM_E_INVALID = -1, SWM_E_UNSUPPORTED = -2, &
                             SWM_E_CUDA = -3, SWM_E_NOMEM = -4, SWM_E_DEVICE = -5, SWM_E_IO = -6
integer(c_int), parameter :: SWM_FP64_PLAIN = 0, SWM_FP32_FUSED = 1
integer(c_int), parameter :: SWM_BOX_AUTO = 0, SWM_BOX_STRIP = 1, SWM_BOX_WIDEST = 2
integer(c_int), parameter :: SWM_SYNC_STATIC_MAX_N = 1024
integer(c_int), parameter :: SWM_GRID_AH = 0, SWM_GRID_C = 1
integer(c_int), parameter :: SWM_MESH_P = 0, SWM_MESH_U = 1, SWM_MESH_V = 2, SWM_MESH_Q = 3

! struct swm_config
type, bind(c) :: swm_config
    integer(c_int) :: N, sbp_order
    real(c_double) :: radius, grav, omega, rotation_axis(3)
    integer(c_int) :: precision, device
end type swm_config

interface
    ! ---------------------------------------------------------- construction
    integer(c_int) function swm_ctx_create(cfg, ctx) bind(c, name="swm_ctx_create")
        import :: c_int, c_ptr, swm_config
        type(swm_config), intent(in) :: cfg
        type(c_ptr), intent(out) :: ctx
    end function swm_ctx_create
    integer(c_int) function swm_ctx_create_named(cfg, div_op_name, grad_op_name, curl_op_name, &
            coriolis_op_name, KE_op_name, co2contra_op_name, massflux_op_name, quadrature_name, &
            ctx) bind(c, name="swm_ctx_create_named")
        import :: c_int, c_ptr, c_char, swm_config
        type(swm_config), intent(in) :: cfg
        character(kind=c_char), intent(in) :: div_op_name(*), grad_op_name(*), curl_op_name(*), &
                                              coriolis_op_name(*), KE_op_name(*), &
                                              co2contra_op_name(*), massflux_op_name(*), &
                                              quadrature_name(*)
        type(c_ptr), intent(out) :: ctx
    end function swm_ctx_create_named
    subroutine swm_ctx_destroy(ctx) bind(c, name="swm_ctx_destroy")
        import :: c_ptr
        type(c_ptr), value :: ctx
    end subroutine swm_ctx_destroy
    type(c_ptr) function swm_last_error(ctx) bind(c, name="swm_last_error")
        import :: c_ptr
        type(c_ptr), value :: ctx
    end function swm_last_error
    integer(c_int) function swm_ctx_synchronize(ctx) bind(c, name="swm_ctx_synchronize")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
    end function swm_ctx_synchronize
    type(c_ptr) function swm_ctx_stream(ctx) bind(c, name="swm_ctx_stream")
        import :: c_ptr
        type(c_ptr), value :: ctx
    end function swm_ctx_stream
    integer(c_size_t) function swm_ctx_npts(ctx) bind(c, name="swm_ctx_npts")
        import :: c_size_t, c_ptr
        type(c_ptr), value :: ctx
    end function swm_ctx_npts
    integer(c_int) function swm_ctx_grid(ctx) bind(c, name="swm_ctx_grid")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
    end function swm_ctx_grid
    integer(c_int) function swm_mesh_dims(ctx, mesh, nx, ny) bind(c, name="swm_mesh_dims")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
        integer(c_int), value :: mesh
        integer(c_int), intent(out) :: nx, ny
    end function swm_mesh_dims
    integer(c_int) function swm_set_orography(ctx, h_surf) bind(c, name="swm_set_orography")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx
        real(c_double), intent(in) :: h_surf(*)
    end function swm_set_orography

    ! ---------------------------------------------------------- state vector
    integer(c_int) function swm_state_create(ctx, s) bind(c, name="swm_state_create")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
        type(c_ptr), intent(out) :: s
    end function swm_state_create
    integer(c_int) function swm_state_create_similar(ctx, src, s) bind(c, name="swm_state_create_similar")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, src
        type(c_ptr), intent(out) :: s
    end function swm_state_create_similar
    subroutine swm_state_free(s) bind(c, name="swm_state_free")
        import :: c_ptr
        type(c_ptr), value :: s
    end subroutine swm_state_free
    integer(c_int) function swm_state_upload(ctx, s, h, u, v) bind(c, name="swm_state_upload")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s
        real(c_double), intent(in) :: h(*), u(*), v(*)
    end function swm_state_upload
    integer(c_int) function swm_state_download(ctx, s, h, u, v) bind(c, name="swm_state_download")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s
        real(c_double), intent(out) :: h(*), u(*), v(*)
    end function swm_state_download
    ! The asynchronous transfers read / write the host arrays after the call
    ! returns, so they take their addresses (c_loc of contiguous target
    ! arrays): an assumed-size dummy could be a temporary copy.
    integer(c_int) function swm_state_upload_async(ctx, s, h, u, v) bind(c, name="swm_state_upload_async")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, s, h, u, v
    end function swm_state_upload_async
    integer(c_int) function swm_state_download_async(ctx, s, h, u, v) bind(c, name="swm_state_download_async")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, s, h, u, v
    end function swm_state_download_async
    integer(c_int) function swm_assign_s1(ctx, s, s1) bind(c, name="swm_assign_s1")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s
        real(c_double), value :: s1
    end function swm_assign_s1
    integer(c_int) function swm_assign_s1v1(ctx, s, s1, v1) bind(c, name="swm_assign_s1v1")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s, v1
        real(c_double), value :: s1
    end function swm_assign_s1v1
    integer(c_int) function swm_assign_s1v1s2v2(ctx, s, s1, v1, s2, v2) bind(c, name="swm_assign_s1v1s2v2")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s, v1, v2
        real(c_double), value :: s1, s2
    end function swm_assign_s1v1s2v2
    integer(c_int) function swm_update_s1v1(ctx, s, s1, v1) bind(c, name="swm_update_s1v1")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s, v1
        real(c_double), value :: s1
    end function swm_update_s1v1
    integer(c_int) function swm_update_s1v1s2v2(ctx, s, s1, v1, s2, v2) bind(c, name="swm_update_s1v1s2v2")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s, v1, v2
        real(c_double), value :: s1, s2
    end function swm_update_s1v1s2v2
    integer(c_int) function swm_dot(ctx, a, b, res) bind(c, name="swm_dot")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, a, b
        real(c_double), intent(out) :: res
    end function swm_dot
    integer(c_int) function swm_norm2(ctx, a, res) bind(c, name="swm_norm2")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, a
        real(c_double), intent(out) :: res
    end function swm_norm2

    ! ---------------------------------------------------------- operator and time scheme
    integer(c_int) function swm_apply(ctx, vout, vin) bind(c, name="swm_apply")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, vout, vin
    end function swm_apply
    integer(c_int) function swm_apply_unfused(ctx, vout, vin) bind(c, name="swm_apply_unfused")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, vout, vin
    end function swm_apply_unfused
    integer(c_int) function swm_rk4_step(ctx, v0, dt, nsteps) bind(c, name="swm_rk4_step")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, v0
        real(c_double), value :: dt
        integer(c_int), value :: nsteps
    end function swm_rk4_step

    ! ---------------------------------------------------------- hyperdiffusion split step
    integer(c_int) function swm_diffusion_set(ctx, hordiff_uv_name, uv_diff_coeff, hordiff_h_name, &
            h_diff_coeff) bind(c, name="swm_diffusion_set")
        import :: c_int, c_ptr, c_char, c_double
        type(c_ptr), value :: ctx
        character(kind=c_char), intent(in) :: hordiff_uv_name(*), hordiff_h_name(*)
        real(c_double), value :: uv_diff_coeff, h_diff_coeff
    end function swm_diffusion_set
    integer(c_int) function swm_apply_diffusion(ctx, vout, vin) bind(c, name="swm_apply_diffusion")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, vout, vin
    end function swm_apply_diffusion
    integer(c_int) function swm_diffusion_step(ctx, v0, dt, nsteps) bind(c, name="swm_diffusion_step")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, v0
        real(c_double), value :: dt
        integer(c_int), value :: nsteps
    end function swm_diffusion_step
    integer(c_int) function swm_model_step(ctx, v0, dt, nsteps) bind(c, name="swm_model_step")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, v0
        real(c_double), value :: dt
        integer(c_int), value :: nsteps
    end function swm_model_step
    integer(c_int) function swm_laplace(ctx, fout, fin, narrow_order) bind(c, name="swm_laplace")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, fout, fin
        integer(c_int), value :: narrow_order
    end function swm_laplace
    integer(c_int) function swm_diagnostics(ctx, v, diag) bind(c, name="swm_diagnostics")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, v
        real(c_double), intent(out) :: diag(7)
    end function swm_diagnostics

    ! ---------------------------------------------------------- fields and single operators
    integer(c_int) function swm_field_create(ctx, f) bind(c, name="swm_field_create")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
        type(c_ptr), intent(out) :: f
    end function swm_field_create
    integer(c_int) function swm_field_create_mesh(ctx, mesh, f) bind(c, name="swm_field_create_mesh")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
        integer(c_int), value :: mesh
        type(c_ptr), intent(out) :: f
    end function swm_field_create_mesh
    subroutine swm_field_free(f) bind(c, name="swm_field_free")
        import :: c_ptr
        type(c_ptr), value :: f
    end subroutine swm_field_free
    integer(c_int) function swm_field_upload(ctx, f, host) bind(c, name="swm_field_upload")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, f
        real(c_double), intent(in) :: host(*)
    end function swm_field_upload
    integer(c_int) function swm_field_download(ctx, f, host) bind(c, name="swm_field_download")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, f
        real(c_double), intent(out) :: host(*)
    end function swm_field_download
    integer(c_int) function swm_op_co2contra(ctx, ut, vt, u, v) bind(c, name="swm_op_co2contra")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, ut, vt, u, v
    end function swm_op_co2contra
    integer(c_int) function swm_op_massflux(ctx, hu, hv, h, ut, vt) bind(c, name="swm_op_massflux")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, hu, hv, h, ut, vt
    end function swm_op_massflux
    integer(c_int) function swm_op_ke(ctx, ke, u, v, ut, vt) bind(c, name="swm_op_ke")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, ke, u, v, ut, vt
    end function swm_op_ke
    integer(c_int) function swm_op_grad(ctx, gx, gy, f) bind(c, name="swm_op_grad")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, gx, gy, f
    end function swm_op_grad
    integer(c_int) function swm_op_div(ctx, div, u, v) bind(c, name="swm_op_div")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, div, u, v
    end function swm_op_div
    integer(c_int) function swm_op_curl(ctx, curl, u, v) bind(c, name="swm_op_curl")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, curl, u, v
    end function swm_op_curl
    integer(c_int) function swm_op_coriolis(ctx, cor_u, cor_v, hu, hv, h, curl) bind(c, name="swm_op_coriolis")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, cor_u, cor_v, hu, hv, h, curl
    end function swm_op_coriolis
    integer(c_int) function swm_op_grad_perp(ctx, gu, gv, w) bind(c, name="swm_op_grad_perp")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, gu, gv, w
    end function swm_op_grad_perp
    integer(c_int) function swm_op_contra2co(ctx, u, v, ut, vt) bind(c, name="swm_op_contra2co")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, u, v, ut, vt
    end function swm_op_contra2co
    integer(c_int) function swm_op_grad_a2_ecs(ctx, gx, gy, f) bind(c, name="swm_op_grad_a2_ecs")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, gx, gy, f
    end function swm_op_grad_a2_ecs
    integer(c_int) function swm_halo_ecs_o(ctx, f, halo_width, ext) bind(c, name="swm_halo_ecs_o")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, f
        integer(c_int), value :: halo_width
        real(c_double), intent(out) :: ext(*)
    end function swm_halo_ecs_o
    integer(c_int) function swm_op_div_a2_ecs(ctx, div, u, v) bind(c, name="swm_op_div_a2_ecs")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, div, u, v
    end function swm_op_div_a2_ecs
    integer(c_int) function swm_op_grad_c2_ecs(ctx, gx, gy, f) bind(c, name="swm_op_grad_c2_ecs")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, gx, gy, f
    end function swm_op_grad_c2_ecs
    integer(c_int) function swm_halo_ecs_xy(ctx, f, halo_width, ext) bind(c, name="swm_halo_ecs_xy")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, f
        integer(c_int), value :: halo_width
        real(c_double), intent(out) :: ext(*)
    end function swm_halo_ecs_xy
    integer(c_int) function swm_laplace_ch(ctx, out, in, order) bind(c, name="swm_laplace_ch")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, out, in
        integer(c_int), value :: order
    end function swm_laplace_ch
    integer(c_int) function swm_halo_ecs_a_vec(ctx, u, v, halo_width, ext_u, ext_v) bind(c, name="swm_halo_ecs_a_vec")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, u, v
        integer(c_int), value :: halo_width
        real(c_double), intent(out) :: ext_u(*), ext_v(*)
    end function swm_halo_ecs_a_vec
    integer(c_int) function swm_sync_scalar(ctx, f) bind(c, name="swm_sync_scalar")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, f
    end function swm_sync_scalar
    integer(c_int) function swm_sync_vector_cov(ctx, gx, gy) bind(c, name="swm_sync_vector_cov")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, gx, gy
    end function swm_sync_vector_cov
    integer(c_int) function swm_quadrature_mass(ctx, f, res) bind(c, name="swm_quadrature_mass")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, f
        real(c_double), intent(out) :: res
    end function swm_quadrature_mass

    ! ---------------------------------------------------------- kernel timing
    integer(c_int) function swm_timing_enable(ctx, on) bind(c, name="swm_timing_enable")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
        integer(c_int), value :: on
    end function swm_timing_enable
    integer(c_int) function swm_timing_read(ctx, stage_ms, stage_launches, edge_ms, edge_launches) &
            bind(c, name="swm_timing_read")
        import :: c_int, c_ptr, c_double, c_long
        type(c_ptr), value :: ctx
        real(c_double), intent(out) :: stage_ms, edge_ms
        integer(c_long), intent(out) :: stage_launches, edge_launches
    end function swm_timing_read

    ! ---------------------------------------------------------- tangent-linear and adjoint
    integer(c_int) function swm_apply_tl(ctx, y, dx, dk) bind(c, name="swm_apply_tl")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, y, dx, dk
    end function swm_apply_tl
    integer(c_int) function swm_apply_ad(ctx, y, lk, lx) bind(c, name="swm_apply_ad")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, y, lk, lx
    end function swm_apply_ad
    integer(c_int) function swm_rk4_tl(ctx, x, dx, dt) bind(c, name="swm_rk4_tl")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, x, dx
        real(c_double), value :: dt
    end function swm_rk4_tl
    integer(c_int) function swm_rk4_ad(ctx, x, lx, dt) bind(c, name="swm_rk4_ad")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, x, lx
        real(c_double), value :: dt
    end function swm_rk4_ad
    integer(c_int) function swm_adjoint_create(ctx, nsteps, nsnap, dt, adj) bind(c, name="swm_adjoint_create")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx
        integer(c_int), value :: nsteps, nsnap
        real(c_double), value :: dt
        type(c_ptr), intent(out) :: adj
    end function swm_adjoint_create
    subroutine swm_adjoint_destroy(adj) bind(c, name="swm_adjoint_destroy")
        import :: c_ptr
        type(c_ptr), value :: adj
    end subroutine swm_adjoint_destroy
    integer(c_int) function swm_adjoint_forward(adj, x0, xT) bind(c, name="swm_adjoint_forward")
        import :: c_int, c_ptr
        type(c_ptr), value :: adj, x0, xT
    end function swm_adjoint_forward
    integer(c_int) function swm_adjoint_backward(adj, lambda) bind(c, name="swm_adjoint_backward")
        import :: c_int, c_ptr
        type(c_ptr), value :: adj, lambda
    end function swm_adjoint_backward
    integer(c_int) function swm_adjoint_counts(adj, forward_steps, adjoint_steps, planned_forward_steps) &
            bind(c, name="swm_adjoint_counts")
        import :: c_int, c_ptr, c_long
        type(c_ptr), value :: adj
        integer(c_long), intent(out) :: forward_steps, adjoint_steps, planned_forward_steps
    end function swm_adjoint_counts
    ! device arrays (c_ptr device addresses) in the host layout
    integer(c_int) function swm_state_upload_device(ctx, s, h, u, v) bind(c, name="swm_state_upload_device")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, s, h, u, v
    end function swm_state_upload_device
    integer(c_int) function swm_state_download_device(ctx, s, h, u, v) bind(c, name="swm_state_download_device")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, s, h, u, v
    end function swm_state_download_device
    integer(c_int) function swm_quadrature_weights(ctx, w_host) bind(c, name="swm_quadrature_weights")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx
        real(c_double), intent(out) :: w_host(*)
    end function swm_quadrature_weights

    ! ---------------------------------------------------------- ensembles
    integer(c_int) function swm_ensemble_create(base, nmembers, member_N, member_dt, ens) &
            bind(c, name="swm_ensemble_create")
        import :: c_int, c_ptr, c_double, swm_config
        type(swm_config), intent(in) :: base
        integer(c_int), value :: nmembers
        integer(c_int), intent(in) :: member_N(*)
        real(c_double), intent(in) :: member_dt(*)
        type(c_ptr), intent(out) :: ens
    end function swm_ensemble_create
    subroutine swm_ensemble_destroy(ens) bind(c, name="swm_ensemble_destroy")
        import :: c_ptr
        type(c_ptr), value :: ens
    end subroutine swm_ensemble_destroy
    type(c_ptr) function swm_ensemble_last_error(ens) bind(c, name="swm_ensemble_last_error")
        import :: c_ptr
        type(c_ptr), value :: ens
    end function swm_ensemble_last_error
    integer(c_int) function swm_ensemble_size(ens) bind(c, name="swm_ensemble_size")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
    end function swm_ensemble_size
    integer(c_int) function swm_ensemble_member(ens, m, ctx, state) bind(c, name="swm_ensemble_member")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
        integer(c_int), value :: m
        type(c_ptr), intent(out) :: ctx, state
    end function swm_ensemble_member
    integer(c_int) function swm_ensemble_upload(ens, m, h, u, v) bind(c, name="swm_ensemble_upload")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ens
        integer(c_int), value :: m
        real(c_double), intent(in) :: h(*), u(*), v(*)
    end function swm_ensemble_upload
    integer(c_int) function swm_ensemble_download(ens, m, h, u, v) bind(c, name="swm_ensemble_download")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ens
        integer(c_int), value :: m
        real(c_double), intent(out) :: h(*), u(*), v(*)
    end function swm_ensemble_download
    integer(c_int) function swm_ensemble_diagnostics(ens, m, diag) bind(c, name="swm_ensemble_diagnostics")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ens
        integer(c_int), value :: m
        real(c_double), intent(out) :: diag(7)
    end function swm_ensemble_diagnostics
    integer(c_int) function swm_ensemble_step(ens, nsteps) bind(c, name="swm_ensemble_step")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
        integer(c_int), value :: nsteps
    end function swm_ensemble_step
    integer(c_int) function swm_ensemble_synchronize(ens) bind(c, name="swm_ensemble_synchronize")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
    end function swm_ensemble_synchronize
    type(c_ptr) function swm_ensemble_stream(ens) bind(c, name="swm_ensemble_stream")
        import :: c_ptr
        type(c_ptr), value :: ens
    end function swm_ensemble_stream
    integer(c_int) function swm_ensemble_set_shape(ens, seg_rows, grid) bind(c, name="swm_ensemble_set_shape")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
        integer(c_int), value :: seg_rows, grid
    end function swm_ensemble_set_shape
    integer(c_int) function swm_ensemble_set_width(ens, cols) bind(c, name="swm_ensemble_set_width")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
        integer(c_int), value :: cols
    end function swm_ensemble_set_width
    integer(c_int) function swm_ensemble_get_width(ens, cols) bind(c, name="swm_ensemble_get_width")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
        integer(c_int), intent(out) :: cols
    end function swm_ensemble_get_width
    integer(c_int) function swm_ensemble_get_shape(ens, seg_rows, grid, nunits) bind(c, name="swm_ensemble_get_shape")
        import :: c_int, c_ptr
        type(c_ptr), value :: ens
        integer(c_int), intent(out) :: seg_rows, grid, nunits
    end function swm_ensemble_get_shape
    integer(c_int) function swm_ensemble_tune(ens, steps, seg_rows_out, grid_out, ms_per_step_out) &
            bind(c, name="swm_ensemble_tune")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ens
        integer(c_int), value :: steps
        integer(c_int), intent(out) :: seg_rows_out, grid_out
        real(c_double), intent(out) :: ms_per_step_out
    end function swm_ensemble_tune

    ! ---------------------------------------------------------- scalar sync, static scratch
    integer(c_int) function swm_sync_scalar_static(ctx, f) bind(c, name="swm_sync_scalar_static")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, f
    end function swm_sync_scalar_static

    ! ---------------------------------------------------------- lat-lon and paneled output
    integer(c_int) function swm_latlon_create(ctx, nlon, nlat, interp_type, components_type, r) &
            bind(c, name="swm_latlon_create")
        import :: c_int, c_ptr, c_char
        type(c_ptr), value :: ctx
        integer(c_int), value :: nlon, nlat
        character(kind=c_char), intent(in) :: interp_type(*), components_type(*)
        type(c_ptr), intent(out) :: r
    end function swm_latlon_create
    subroutine swm_latlon_destroy(r) bind(c, name="swm_latlon_destroy")
        import :: c_ptr
        type(c_ptr), value :: r
    end subroutine swm_latlon_destroy
    integer(c_int) function swm_latlon_regrid_field(ctx, r, f, fout) bind(c, name="swm_latlon_regrid_field")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, r, f
        real(c_double), intent(out) :: fout(*)
    end function swm_latlon_regrid_field
    integer(c_int) function swm_latlon_regrid_vector(ctx, r, u, v, uo, vo) bind(c, name="swm_latlon_regrid_vector")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, r, u, v
        real(c_double), intent(out) :: uo(*), vo(*)
    end function swm_latlon_regrid_vector
    ! h, u, v: c_loc of the output arrays, or c_null_ptr to skip one
    integer(c_int) function swm_latlon_regrid_state(ctx, r, s, h, u, v) bind(c, name="swm_latlon_regrid_state")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx, r, s, h, u, v
    end function swm_latlon_regrid_state
    ! file names: trim(name)//c_null_char; an empty name (c_null_char alone) skips that file
    integer(c_int) function swm_latlon_write(ctx, r, s, h_file, u_file, v_file, rec_num) &
            bind(c, name="swm_latlon_write")
        import :: c_int, c_ptr, c_char
        type(c_ptr), value :: ctx, r, s
        character(kind=c_char), intent(in) :: h_file(*), u_file(*), v_file(*)
        integer(c_int), value :: rec_num
    end function swm_latlon_write
    integer(c_int) function swm_paneled_write(ctx, s, component, file, rec_num) bind(c, name="swm_paneled_write")
        import :: c_int, c_ptr, c_char
        type(c_ptr), value :: ctx, s
        integer(c_int), value :: component, rec_num
        character(kind=c_char), intent(in) :: file(*)
    end function swm_paneled_write

    ! ---------------------------------------------------------- launch-shape tuning
    integer(c_int) function swm_tune_stage(ctx, s, dt, steps, cols_out, seg_rows_out, grid_out, box_out, ms_out) &
            bind(c, name="swm_tune_stage")
        import :: c_int, c_ptr, c_double
        type(c_ptr), value :: ctx, s
        real(c_double), value :: dt
        integer(c_int), value :: steps
        integer(c_int), intent(out) :: cols_out, seg_rows_out, grid_out, box_out
        real(c_double), intent(out) :: ms_out
    end function swm_tune_stage
    integer(c_int) function swm_get_stage_shape(ctx, cols, seg_rows, grid, box, nunits) &
            bind(c, name="swm_get_stage_shape")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
        integer(c_int), intent(out) :: cols, seg_rows, grid, box, nunits
    end function swm_get_stage_shape
    integer(c_int) function swm_set_stage_shape(ctx, cols, seg_rows, grid, box) bind(c, name="swm_set_stage_shape")
        import :: c_int, c_ptr
        type(c_ptr), value :: ctx
        integer(c_int), value :: cols, seg_rows, grid, box
    end function swm_set_stage_shape
    integer(c_int) function swm_work_split(N, sbp_order, cols, target_units, seg_rows, units_out, max_units, &
            nunits) bind(c, name="swm_work_split")
        import :: c_int
        integer(c_int), value :: N, sbp_order, cols, target_units, seg_rows, max_units
        integer(c_int), intent(out) :: units_out(*), nunits
    end function swm_work_split

    ! ---------------------------------------------------------- checkpoint / resume
    integer(c_int) function swm_state_save(ctx, s, path, time) bind(c, name="swm_state_save")
        import :: c_int, c_ptr, c_char, c_double
        type(c_ptr), value :: ctx, s
        character(kind=c_char), intent(in) :: path(*)
        real(c_double), value :: time
    end function swm_state_save
    integer(c_int) function swm_state_load(ctx, s, path, time) bind(c, name="swm_state_load")
        import :: c_int, c_ptr, c_char, c_double
        type(c_ptr), value :: ctx, s
        character(kind=c_char), intent(in) :: path(*)
        real(c_double), intent(out) :: time
    end function swm_state_load
end interface

contains

! The NUL-terminated message of the last failure on ctx (c_null_ptr: the
! last failure without a context) as a Fortran string.
function swm_error_message(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: p(:)
    type(c_ptr) :: cp
    integer :: k, n

    interface
        integer(c_size_t) function c_strlen(s) bind(c, name="strlen")
            import :: c_size_t, c_ptr
            type(c_ptr), value :: s
        end function c_strlen
    end interface

    cp = swm_last_error(ctx)
    if (.not. c_associated(cp)) then
        msg = ""
        return
    end if
    n = int(c_strlen(cp))
    call c_f_pointer(cp, p, [n])
    allocate(character(len=n) :: msg)
    do k = 1, n
        msg(k:k) = p(k)
    end do
end function swm_error_message

end module swm_gpu_c
