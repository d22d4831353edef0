! swm_gpu_shim.f90 -- drop-in types for the reference's Fortran plugin
! surface (vvshashkin/cubedsphere_sbp_swm) over the GB300 C-ABI (swm_gpu_c).
!
! The reference's time loop (ts2_mod.f90:143-153, barotropic_inst_mod.f90:
! 163-174) only calls the abstract interfaces below, so it keeps its calls
! when these types replace the CPU ones:
!   stvec_swm_gpu_t     extends stvec_t       (stvec_mod.f90:10-28): every
!                       procedure of stvec_t is overridden; the state lives
!                       on the GPU, (h, u, v) of one context
!   operator_swm_gpu_t  extends operator_t    (operator_mod.f90:11-26):
!                       apply = operator_swm_t%apply (operator_swm_mod.f90:
!                       61-113), get_diagnostics (operator_swm_mod.f90:115-155)
!   operator_swm_diff_gpu_t extends operator_t: apply = operator_swm_diff_t
!                       %apply (operator_swm_diff_mod.f90:25-46)
!   rk4_gpu_t           extends timescheme_t  (timescheme_mod.f90:9-28): the
!                       fused RK4 step (rk4_mod.f90:20-42) on GPU states with
!                       the GPU operator; any other operator/state pair runs
!                       the same RK4 through apply/assign/update
!   explicit_Eul1_gpu_t extends timescheme_t: explicit_Eul1_t%step
!                       (explicit_Eul1_mod.f90:20-30), fused on the GPU for the
!                       GPU diffusion operator
! The domain_t argument of the interfaces is unused: the context holds the
! grid, metric and SBP operators it was created with.  A failing call ends
! the run through parcomm_global%abort with the library's message, as the
! reference's own errors do (parcomm_mod.f90:73-83).
!
! States are handles: copy them with copy_to / create_similar + assign, not
! with intrinsic assignment (which would copy the handle), and release them
! with %free.
module swm_gpu_shim
use iso_c_binding
use swm_gpu_c
use stvec_mod,      only : stvec_t
use operator_mod,   only : operator_t
use timescheme_mod, only : timescheme_t
use domain_mod,     only : domain_t
use parcomm_mod,    only : parcomm_global
use key_value_mod,  only : key_value_r8_t
implicit none

private
public :: stvec_swm_gpu_t, operator_swm_gpu_t, operator_swm_diff_gpu_t, rk4_gpu_t, &
          explicit_Eul1_gpu_t, create_swm_gpu_operator, create_swm_gpu_stvec, &
          create_swm_gpu_diff_operator

type, extends(stvec_t) :: stvec_swm_gpu_t
    type(c_ptr) :: ctx = c_null_ptr    ! the operator's context (not owned)
    type(c_ptr) :: s   = c_null_ptr    ! swm_state handle (owned)
contains
    procedure, public :: copy_to         => gpu_copy_to
    procedure, public :: create_similar  => gpu_create_similar
    procedure, public :: update_s1v1     => gpu_update_s1v1
    procedure, public :: update_s1v1s2v2 => gpu_update_s1v1s2v2
    procedure, public :: assign_s1       => gpu_assign_s1
    procedure, public :: assign_s1v1     => gpu_assign_s1v1
    procedure, public :: assign_s1v1s2v2 => gpu_assign_s1v1s2v2
    procedure, public :: algebraic_norm2 => gpu_algebraic_norm2
    procedure, public :: algebraic_dot   => gpu_algebraic_dot
    procedure, public :: upload          => gpu_upload     ! host tile arrays -> device
    procedure, public :: download        => gpu_download   ! device -> host tile arrays
    procedure, public :: free            => gpu_free
end type stvec_swm_gpu_t

type, extends(operator_t) :: operator_swm_gpu_t
    type(c_ptr) :: ctx = c_null_ptr    ! swm_ctx handle (owned)
contains
    procedure, public :: apply           => gpu_apply
    procedure, public :: get_diagnostics => gpu_get_diagnostics
    procedure, public :: destroy         => gpu_operator_destroy
end type operator_swm_gpu_t

type, extends(operator_t) :: operator_swm_diff_gpu_t
    type(c_ptr) :: ctx = c_null_ptr    ! the model operator's context (not owned)
contains
    procedure, public :: apply => gpu_apply_diffusion
end type operator_swm_diff_gpu_t

type, extends(timescheme_t) :: rk4_gpu_t
    ! work vectors of the generic path (other operators / states), created on
    ! first use as rk4_t's are (timescheme_factory_mod.f90:42-59)
    class(stvec_t), allocatable :: k1, k2, k3, k4, y
contains
    procedure, public :: step => gpu_rk4_step
end type rk4_gpu_t

type, extends(timescheme_t) :: explicit_Eul1_gpu_t
    class(stvec_t), allocatable :: tendency
contains
    procedure, public :: step => gpu_eul1_step
end type explicit_Eul1_gpu_t

contains

! ------------------------------------------------------------------ helpers
subroutine check(rc, ctx, what)
    integer(c_int),   intent(in) :: rc
    type(c_ptr),      intent(in) :: ctx
    character(len=*), intent(in) :: what

    if (rc /= SWM_OK) call parcomm_global%abort("swm_gpu " // what // ": " // swm_error_message(ctx))
end subroutine check

! The GPU handle of a state given through the abstract interface.
function handle_of(v, what) result(s)
    class(stvec_t),   intent(in) :: v
    character(len=*), intent(in) :: what
    type(c_ptr) :: s

    s = c_null_ptr
    select type (v)
    class is (stvec_swm_gpu_t)
        s = v%s
    class default
        call parcomm_global%abort("swm_gpu " // what // ": the state is not a stvec_swm_gpu_t")
    end select
end function handle_of

! ------------------------------------------------------------------ construction
! create_domain + create_swm_operator + create_timescheme in one context
! (domain_factory_mod.f90:44-136, operator_swm_factory_mod.f90:43-131); the
! operator names are the &shallow_water_model namelist's (config_swm_mod.f90
! :70-104), e.g. "divergence_ah42_sbp", "gradient_ah42_sbp_ecs",
! "curl_divergence_ah42_sbp", "coriolis_colocated", "KE_colocated",
! "co2contra_colocated", "massflux_colocated", "SBP_Ah42_quadrature".
subroutine create_swm_gpu_operator(op, N, sbp_order, radius, grav, omega, rotation_axis, precision, &
                                   device, div_op_name, grad_op_name, curl_op_name, coriolis_op_name, &
                                   KE_op_name, co2contra_op_name, massflux_op_name, quadrature_name)
    type(operator_swm_gpu_t), intent(out) :: op
    integer,                  intent(in)  :: N, sbp_order, precision, device
    real(kind=8),             intent(in)  :: radius, grav, omega, rotation_axis(3)
    character(len=*),         intent(in)  :: div_op_name, grad_op_name, curl_op_name, coriolis_op_name, &
                                             KE_op_name, co2contra_op_name, massflux_op_name, &
                                             quadrature_name
    type(swm_config) :: cfg
    integer(c_int)   :: rc

    cfg%N = int(N, c_int)
    cfg%sbp_order = int(sbp_order, c_int)
    cfg%radius = radius
    cfg%grav = grav
    cfg%omega = omega
    cfg%rotation_axis = rotation_axis
    cfg%precision = int(precision, c_int)
    cfg%device = int(device, c_int)
    rc = swm_ctx_create_named(cfg, trim(div_op_name)//c_null_char, trim(grad_op_name)//c_null_char, &
                              trim(curl_op_name)//c_null_char, trim(coriolis_op_name)//c_null_char, &
                              trim(KE_op_name)//c_null_char, trim(co2contra_op_name)//c_null_char, &
                              trim(massflux_op_name)//c_null_char, trim(quadrature_name)//c_null_char, &
                              op%ctx)
    call check(rc, c_null_ptr, "create_swm_gpu_operator")
end subroutine create_swm_gpu_operator

! create_stvec_swm (stvec_swm_factory_mod.f90:22-24): a zero state of the context
subroutine create_swm_gpu_stvec(v, op)
    class(stvec_t), allocatable, intent(out) :: v
    type(operator_swm_gpu_t),    intent(in)  :: op
    type(c_ptr)    :: s
    integer(c_int) :: rc

    rc = swm_state_create(op%ctx, s)
    call check(rc, op%ctx, "create_swm_gpu_stvec")
    allocate(stvec_swm_gpu_t :: v)
    select type (v)
    type is (stvec_swm_gpu_t)
        v%ctx = op%ctx
        v%s = s
    end select
end subroutine create_swm_gpu_stvec

! create_swm_diff_operator (operator_swm_diff_factory_mod.f90:27-30) with the
! namelist's hordiff_uv_name, uv_diff_coeff, hordiff_h_name, h_diff_coeff
subroutine create_swm_gpu_diff_operator(dop, op, hordiff_uv_name, uv_diff_coeff, hordiff_h_name, &
                                        h_diff_coeff)
    type(operator_swm_diff_gpu_t), intent(out) :: dop
    type(operator_swm_gpu_t),      intent(in)  :: op
    character(len=*),              intent(in)  :: hordiff_uv_name, hordiff_h_name
    real(kind=8),                  intent(in)  :: uv_diff_coeff, h_diff_coeff
    integer(c_int) :: rc

    rc = swm_diffusion_set(op%ctx, trim(hordiff_uv_name)//c_null_char, uv_diff_coeff, &
                           trim(hordiff_h_name)//c_null_char, h_diff_coeff)
    call check(rc, op%ctx, "create_swm_gpu_diff_operator")
    dop%ctx = op%ctx
end subroutine create_swm_gpu_diff_operator

subroutine gpu_operator_destroy(this)
    class(operator_swm_gpu_t), intent(inout) :: this

    if (c_associated(this%ctx)) call swm_ctx_destroy(this%ctx)
    this%ctx = c_null_ptr
end subroutine gpu_operator_destroy

! ------------------------------------------------------------------ stvec_t
subroutine gpu_copy_to(this, destination)
    class(stvec_swm_gpu_t),      intent(in)    :: this
    class(stvec_t), allocatable, intent(inout) :: destination
    integer(c_int) :: rc

    call this%create_similar(destination)
    select type (destination)
    type is (stvec_swm_gpu_t)
        rc = swm_assign_s1v1(this%ctx, destination%s, 1.0_c_double, this%s)
        call check(rc, this%ctx, "copy_to")
    end select
end subroutine gpu_copy_to

subroutine gpu_create_similar(this, destination)
    class(stvec_swm_gpu_t),      intent(in)    :: this
    class(stvec_t), allocatable, intent(inout) :: destination
    type(c_ptr)    :: s
    integer(c_int) :: rc

    rc = swm_state_create_similar(this%ctx, this%s, s)
    call check(rc, this%ctx, "create_similar")
    if (allocated(destination)) deallocate(destination)
    allocate(stvec_swm_gpu_t :: destination)
    select type (destination)
    type is (stvec_swm_gpu_t)
        destination%ctx = this%ctx
        destination%s = s
    end select
end subroutine gpu_create_similar

subroutine gpu_update_s1v1(this, scalar1, v1, domain)
    class(stvec_swm_gpu_t), intent(inout) :: this
    real(kind=8),           intent(in)    :: scalar1
    class(stvec_t),         intent(in)    :: v1
    class(domain_t),        intent(in)    :: domain

    call check(swm_update_s1v1(this%ctx, this%s, scalar1, handle_of(v1, "update_s1v1")), &
               this%ctx, "update_s1v1")
end subroutine gpu_update_s1v1

subroutine gpu_update_s1v1s2v2(this, scalar1, v1, scalar2, v2, domain)
    class(stvec_swm_gpu_t), intent(inout) :: this
    real(kind=8),           intent(in)    :: scalar1, scalar2
    class(stvec_t),         intent(in)    :: v1, v2
    class(domain_t),        intent(in)    :: domain

    call check(swm_update_s1v1s2v2(this%ctx, this%s, scalar1, handle_of(v1, "update_s1v1s2v2"), &
                                   scalar2, handle_of(v2, "update_s1v1s2v2")), &
               this%ctx, "update_s1v1s2v2")
end subroutine gpu_update_s1v1s2v2

subroutine gpu_assign_s1(this, scalar1, domain)
    class(stvec_swm_gpu_t), intent(inout) :: this
    real(kind=8),           intent(in)    :: scalar1
    class(domain_t),        intent(in)    :: domain

    call check(swm_assign_s1(this%ctx, this%s, scalar1), this%ctx, "assign_s1")
end subroutine gpu_assign_s1

subroutine gpu_assign_s1v1(this, scalar1, v1, domain)
    class(stvec_swm_gpu_t), intent(inout) :: this
    real(kind=8),           intent(in)    :: scalar1
    class(stvec_t),         intent(in)    :: v1
    class(domain_t),        intent(in)    :: domain

    call check(swm_assign_s1v1(this%ctx, this%s, scalar1, handle_of(v1, "assign_s1v1")), &
               this%ctx, "assign_s1v1")
end subroutine gpu_assign_s1v1

subroutine gpu_assign_s1v1s2v2(this, scalar1, v1, scalar2, v2, domain)
    class(stvec_swm_gpu_t), intent(inout) :: this
    real(kind=8),           intent(in)    :: scalar1, scalar2
    class(stvec_t),         intent(in)    :: v1, v2
    class(domain_t),        intent(in)    :: domain

    call check(swm_assign_s1v1s2v2(this%ctx, this%s, scalar1, handle_of(v1, "assign_s1v1s2v2"), &
                                   scalar2, handle_of(v2, "assign_s1v1s2v2")), &
               this%ctx, "assign_s1v1s2v2")
end subroutine gpu_assign_s1v1s2v2

function gpu_algebraic_norm2(this, domain) result(norm2)
    class(stvec_swm_gpu_t), intent(in) :: this
    class(domain_t),        intent(in) :: domain
    real(kind=8) :: norm2
    real(c_double) :: r

    call check(swm_norm2(this%ctx, this%s, r), this%ctx, "algebraic_norm2")
    norm2 = r
end function gpu_algebraic_norm2

function gpu_algebraic_dot(this, other, domain) result(dot_product)
    class(stvec_swm_gpu_t), intent(in) :: this
    class(stvec_t),         intent(in) :: other
    class(domain_t),        intent(in) :: domain
    real(kind=8) :: dot_product
    real(c_double) :: r

    call check(swm_dot(this%ctx, this%s, handle_of(other, "algebraic_dot"), r), this%ctx, "algebraic_dot")
    dot_product = r
end function gpu_algebraic_dot

! h, u, v: the reference's tile arrays in panel order, (N+1) x (N+1) x 6 on the
! Ah grid; on the C grid h is N x N x 6, u (N+1) x N x 6, v N x (N+1) x 6
! (swm_mesh_dims)
subroutine gpu_upload(this, h, u, v)
    class(stvec_swm_gpu_t), intent(inout) :: this
    real(kind=8),           intent(in)    :: h(:,:,:), u(:,:,:), v(:,:,:)

    call check(swm_state_upload(this%ctx, this%s, h, u, v), this%ctx, "upload")
end subroutine gpu_upload

subroutine gpu_download(this, h, u, v)
    class(stvec_swm_gpu_t), intent(in)  :: this
    real(kind=8),           intent(out) :: h(:,:,:), u(:,:,:), v(:,:,:)

    call check(swm_state_download(this%ctx, this%s, h, u, v), this%ctx, "download")
end subroutine gpu_download

subroutine gpu_free(this)
    class(stvec_swm_gpu_t), intent(inout) :: this

    if (c_associated(this%s)) call swm_state_free(this%s)
    this%s = c_null_ptr
end subroutine gpu_free

! ------------------------------------------------------------------ operator_t
subroutine gpu_apply(this, vout, vin, domain)
    class(operator_swm_gpu_t), intent(inout) :: this
    class(stvec_t),            intent(inout) :: vout, vin
    type(domain_t),            intent(in)    :: domain

    call check(swm_apply(this%ctx, handle_of(vout, "apply"), handle_of(vin, "apply")), this%ctx, "apply")
end subroutine gpu_apply

function gpu_get_diagnostics(this, v, domain) result(diagnostics)
    class(operator_swm_gpu_t), intent(inout) :: this
    class(stvec_t),            intent(inout) :: v
    type(domain_t),            intent(in)    :: domain
    type(key_value_r8_t) :: diagnostics
    character(len=9), parameter :: names(7) = [character(len=9) :: "hmin", "hmax", "mass", "TE", "KE", &
                                                                  "PE", "Enstrophy"]
    real(c_double) :: d(7)
    integer :: k

    call check(swm_diagnostics(this%ctx, handle_of(v, "get_diagnostics"), d), this%ctx, "get_diagnostics")
    allocate(diagnostics%keys(7))
    allocate(diagnostics%values(7))
    do k = 1, 7
        diagnostics%keys(k)%str = trim(names(k))
        diagnostics%values(k) = d(k)
    end do
end function gpu_get_diagnostics

subroutine gpu_apply_diffusion(this, vout, vin, domain)
    class(operator_swm_diff_gpu_t), intent(inout) :: this
    class(stvec_t),                 intent(inout) :: vout, vin
    type(domain_t),                 intent(in)    :: domain

    call check(swm_apply_diffusion(this%ctx, handle_of(vout, "diffusion apply"), &
                                   handle_of(vin, "diffusion apply")), this%ctx, "diffusion apply")
end subroutine gpu_apply_diffusion

! ------------------------------------------------------------------ timescheme_t
subroutine gpu_rk4_step(this, v0, operator, domain, dt)
    class(rk4_gpu_t),  intent(inout) :: this
    class(stvec_t),    intent(inout) :: v0
    class(operator_t), intent(inout) :: operator
    type(domain_t),    intent(in)    :: domain
    real(kind=8),      intent(in)    :: dt

    select type (operator)
    type is (operator_swm_gpu_t)
        ! the fused step: four stage kernels, replayed as one CUDA graph
        call check(swm_rk4_step(operator%ctx, handle_of(v0, "rk4 step"), dt, 1_c_int), &
                   operator%ctx, "rk4 step")
    class default
        ! any other operator: RK4 through the abstract interfaces, with the
        ! stage combinations in rk4_mod.f90's order
        if (.not. allocated(this%y)) then
            call v0%create_similar(this%k1)
            call v0%create_similar(this%k2)
            call v0%create_similar(this%k3)
            call v0%create_similar(this%k4)
            call v0%create_similar(this%y)
        end if
        call operator%apply(this%k1, v0, domain)
        call this%y%assign(1.0_8, v0, 0.5_8*dt, this%k1, domain)
        call operator%apply(this%k2, this%y, domain)
        call this%y%assign(1.0_8, v0, 0.5_8*dt, this%k2, domain)
        call operator%apply(this%k3, this%y, domain)
        call this%y%assign(1.0_8, v0, dt, this%k3, domain)
        call operator%apply(this%k4, this%y, domain)
        call v0%update(dt/6.0_8, this%k1, dt/3.0_8, this%k2, domain)
        call v0%update(dt/3.0_8, this%k3, dt/6.0_8, this%k4, domain)
    end select
end subroutine gpu_rk4_step

subroutine gpu_eul1_step(this, v0, operator, domain, dt)
    class(explicit_Eul1_gpu_t), intent(inout) :: this
    class(stvec_t),             intent(inout) :: v0
    class(operator_t),          intent(inout) :: operator
    type(domain_t),             intent(in)    :: domain
    real(kind=8),               intent(in)    :: dt

    select type (operator)
    type is (operator_swm_diff_gpu_t)
        ! v0 += dt * D(v0) as one CUDA graph
        call check(swm_diffusion_step(operator%ctx, handle_of(v0, "diffusion step"), dt, 1_c_int), &
                   operator%ctx, "diffusion step")
    class default
        if (.not. allocated(this%tendency)) call v0%create_similar(this%tendency)
        call operator%apply(this%tendency, v0, domain)
        call v0%update(dt, this%tendency, domain)
    end select
end subroutine gpu_eul1_step

end module swm_gpu_shim
