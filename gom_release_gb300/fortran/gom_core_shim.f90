! gom_core_shim.f90 -- the Fortran side of the C ABI in include/gom_core.h: what a maintainer adds
! to GOM_Rv1.1.0/source to run the per-timestep core on a GB300.
!
! Two modules and the replacement subroutines:
!   * gom_core_abi   bind(c) mirrors of gom_dims, gom_params, gom_geom, gom_forcing and gom_status,
!                    field by field in the header's order, the gom_field ids, and interfaces to the
!                    entry points (libgomcore.so);
!   * gom_core_shim  one context per run: gom_gpu_init (call once after prepare_gom, main.f90:47)
!                    creates it from the module arrays of mod_global_variables and uploads the
!                    state; gom_gpu_get copies a field back for the output writers; gom_gpu_step
!                    runs a whole step (main.f90:167-272) as one captured graph;
!   * the subroutines the time loop calls (main.f90:179-272) with the reference's names, each
!     forwarding to its gom_step_* entry point after uploading the host forcing it needs.  Build
!     the model with this file instead of the replaced sources (calculate_bottom_friction.f90,
!     compute_boundary_velocity.f90's core part, solve_nonlinear_advection.f90,
!     solve_momentum_equation.f90, solve_free_surface_equation.f90, solve_velocities.f90,
!     update_vertical_layers_1.f90, calculate_velocity_at_node.f90, solve_transport_equation_v19.f90,
!     calculate_density_full.f90, calculate_density_linear.f90, update_variables.f90) and link
!     gom_release_gb300/_build/libgomcore.so.
!
! Arrays keep their module shapes: the library reads (k, entity) column-major storage with the
! declared lower bounds, so c_loc of the first element is all it needs.  Host arrays are read only
! during a call.  Errors come back as gom_err codes; the shim prints the site, entity and layer
! gom_get_status reports and stops, as the reference's own checks do.
module gom_core_abi
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: GOM_ABI_VERSION = 4
  integer(c_int), parameter :: GOM_OK = 0

  type, bind(c) :: gom_dims
     integer(c_int32_t) :: n_cells
     integer(c_int32_t) :: n_faces
     integer(c_int32_t) :: n_nodes
     integer(c_int32_t) :: n_layers
     integer(c_int32_t) :: max_nb
     integer(c_int32_t) :: n_ob
     integer(c_int32_t) :: n_qb
     integer(c_int32_t) :: n_runs
  end type
  type, bind(c) :: gom_params
     real(c_double) :: gravity
     real(c_double) :: rho_o
     real(c_double) :: msl
     real(c_double) :: dt
     real(c_double) :: theta
     real(c_double) :: adv_onoff_depth
     real(c_double) :: von_karman
     real(c_double) :: cd_const
     real(c_double) :: dry_depth
     real(c_double) :: smagorinsky
     real(c_double) :: ah_0
     real(c_double) :: kh_0
     real(c_double) :: error_tolerance
     real(c_double) :: delta_z_min
     real(c_double) :: denominator_min_for_matrix
     integer(c_int32_t) :: advection_flag
     integer(c_int32_t) :: elm_backtrace_flag
     integer(c_int32_t) :: elm_sub_iter
     integer(c_int32_t) :: elm_min_iter
     integer(c_int32_t) :: elm_max_iter
     integer(c_int32_t) :: bf_flag
     integer(c_int32_t) :: baroclinic_flag
     integer(c_int32_t) :: ana_density
     integer(c_int32_t) :: max_iteration_pcg
     integer(c_int32_t) :: transport_flag
     integer(c_int32_t) :: trans_sub_iter
     integer(c_int32_t) :: h_flux_limiter
     integer(c_int32_t) :: v_flux_limiter
     integer(c_int32_t) :: is_salt
     integer(c_int32_t) :: is_temp
     integer(c_int32_t) :: heat_option
     integer(c_int32_t) :: test_barrier_phantom_blocks
     integer(c_int32_t) :: precision
     integer(c_int32_t) :: turbulence_flag
     integer(c_int32_t) :: transport_solver
     real(c_double) :: pp_h1
     real(c_double) :: pp_h2
     real(c_double) :: pp_vdmax1
     real(c_double) :: pp_vdmax2
     real(c_double) :: pp_vdmin1
     real(c_double) :: pp_vdmin2
     real(c_double) :: pp_tdmin
  end type
  type, bind(c) :: gom_geom
     type(c_ptr) :: x_node
     type(c_ptr) :: y_node
     type(c_ptr) :: h_node
     type(c_ptr) :: adj_cells_at_node
     type(c_ptr) :: adj_cellnum_at_node
     type(c_ptr) :: node_count_each_element
     type(c_ptr) :: adj_nodes_at_node
     type(c_ptr) :: adj_nodenum_at_node
     type(c_ptr) :: bottom_layer_at_node
     type(c_ptr) :: initial_wetdry_node
     type(c_ptr) :: x_cell
     type(c_ptr) :: y_cell
     type(c_ptr) :: h_cell
     type(c_ptr) :: area
     type(c_ptr) :: tri_or_quad
     type(c_ptr) :: nodenum_at_cell
     type(c_ptr) :: facenum_at_cell
     type(c_ptr) :: adj_cellnum_at_cell
     type(c_ptr) :: sign_in_outflow
     type(c_ptr) :: bottom_layer_at_element
     type(c_ptr) :: ob_element_flag
     type(c_ptr) :: qb_element_flag
     type(c_ptr) :: x_face
     type(c_ptr) :: y_face
     type(c_ptr) :: h_face
     type(c_ptr) :: face_length
     type(c_ptr) :: delta_j
     type(c_ptr) :: cos_theta
     type(c_ptr) :: sin_theta
     type(c_ptr) :: cos_theta2
     type(c_ptr) :: sin_theta2
     type(c_ptr) :: adj_cellnum_at_face
     type(c_ptr) :: nodenum_at_face
     type(c_ptr) :: bottom_layer_at_face
     type(c_ptr) :: boundary_type_of_face
     type(c_ptr) :: isflowside3
     type(c_ptr) :: coriolis_factor
     type(c_ptr) :: manning
     type(c_ptr) :: bf_height
     type(c_ptr) :: ob_cell_id
     type(c_ptr) :: qb_cell
     type(c_ptr) :: qb_face
     type(c_ptr) :: z_level
     type(c_ptr) :: delta_z
     type(c_ptr) :: run_cell_start
     type(c_ptr) :: run_face_start
     type(c_ptr) :: run_node_start
     type(c_ptr) :: run_ob_start
  end type
  type, bind(c) :: gom_forcing
     real(c_double) :: elapsed_time
     real(c_double) :: spinup_tide
     real(c_double) :: spinup_baroclinic
     real(c_double) :: reserved
     type(c_ptr) :: eta_at_ob_old
     type(c_ptr) :: eta_at_ob_new
     type(c_ptr) :: q_add
     type(c_ptr) :: wind_stress_normal
     type(c_ptr) :: wind_stress_tangnt
     type(c_ptr) :: gamma_t
     type(c_ptr) :: air_p
     type(c_ptr) :: con_at_ob
     type(c_ptr) :: con_at_qb
     type(c_ptr) :: phi_sw
     type(c_ptr) :: phi_sz
  end type
  type, bind(c) :: gom_status
     integer(c_int32_t) :: code
     integer(c_int32_t) :: site
     integer(c_int32_t) :: entity
     integer(c_int32_t) :: layer
     real(c_double) :: value
     integer(c_int32_t) :: entity_kind
     integer(c_int32_t) :: run
  end type

  type, bind(c) :: gom_series
     integer(c_int32_t) :: n_series
     integer(c_int32_t) :: reserved
     type(c_ptr) :: start
     type(c_ptr) :: time
     type(c_ptr) :: value
  end type

  type, bind(c) :: gom_boundary_series
     real(c_double) :: julian_day
     real(c_double) :: tide_spinup_period
     real(c_double) :: baroclinic_spinup_period
     integer(c_int32_t) :: step
     integer(c_int32_t) :: reference_diff_days
     integer(c_int32_t) :: tide_spinup
     integer(c_int32_t) :: baroclinic_spinup
     integer(c_int32_t) :: q_interp_method
     integer(c_int32_t) :: n_harmonic
     type(c_ptr) :: ob_eta_type
     type(c_ptr) :: ob_harmonic_id
     type(c_ptr) :: ob_eta_id
     type(c_ptr) :: ob_salt_id
     type(c_ptr) :: ob_temp_id
     type(c_ptr) :: qb_q_id
     type(c_ptr) :: qb_salt_id
     type(c_ptr) :: qb_temp_id
     type(c_ptr) :: qb_portion
     type(c_ptr) :: harmonic_start
     type(c_ptr) :: amplitude
     type(c_ptr) :: period_h
     type(c_ptr) :: nodal
     type(c_ptr) :: eq_arg
     type(c_ptr) :: phase
     type(c_ptr) :: phase_shift
     type(gom_series) :: eta
     type(gom_series) :: q
     type(gom_series) :: salt
     type(gom_series) :: temp
     integer(c_int32_t) :: wind_flag
     integer(c_int32_t) :: wind_formular
     integer(c_int32_t) :: wind_spinup
     integer(c_int32_t) :: n_wind
     real(c_double) :: wind_spinup_period
     real(c_double) :: rho_a
     type(c_ptr) :: wind_station_node
     type(gom_series) :: wind_u
     type(gom_series) :: wind_v
     integer(c_int32_t) :: hurricane_flag
     integer(c_int32_t) :: hurricane_read_interval
     real(c_double) :: hurricane_start_jday
     real(c_double) :: hurricane_end_jday
     type(c_ptr) :: hurricane_frames
     integer(c_int32_t) :: hurricane_interp_method
     integer(c_int32_t) :: reserved_hurricane
     real(c_double) :: hurricane_track(6)
     integer(c_int32_t) :: heat_flag
     integer(c_int32_t) :: sol_swr
     integer(c_int32_t) :: n_air
     integer(c_int32_t) :: reserved_heat
     real(c_double) :: fwz_a
     real(c_double) :: fwz_b
     real(c_double) :: fwz_c
     real(c_double) :: wind_height
     real(c_double) :: light_extinction
     real(c_double) :: sol_absorb
     real(c_double) :: sed_water_exchange
     real(c_double) :: t_sed
     real(c_double) :: sed_temp_coeff
     type(c_ptr) :: air_time
     type(c_ptr) :: air_values
     integer(c_int32_t) :: year
     integer(c_int32_t) :: month
     real(c_double) :: lon
     real(c_double) :: lat
  end type

  type, bind(c) :: gom_mesh
     integer(c_int32_t) :: n_nodes
     integer(c_int32_t) :: n_cells
     integer(c_int32_t) :: max_nb
     integer(c_int32_t) :: voronoi
     integer(c_int32_t) :: n_layers
     integer(c_int32_t) :: n_ob
     integer(c_int32_t) :: n_qb
     integer(c_int32_t) :: reserved
     type(c_ptr) :: x_node
     type(c_ptr) :: y_node
     type(c_ptr) :: h_node
     type(c_ptr) :: tri_or_quad
     type(c_ptr) :: nodenum_at_cell
     type(c_ptr) :: z_level
     real(c_double) :: msl
     type(c_ptr) :: ob_nodes
     type(c_ptr) :: qb_nodes
  end type

  type, bind(c) :: gom_mesh_geometry
     integer(c_int32_t) :: face_capacity
     integer(c_int32_t) :: n_faces
     type(c_ptr) :: adj_cells_at_node
     type(c_ptr) :: adj_cellnum_at_node
     type(c_ptr) :: node_count_each_element
     type(c_ptr) :: adj_nodes_at_node
     type(c_ptr) :: adj_nodenum_at_node
     type(c_ptr) :: bottom_layer_at_node
     type(c_ptr) :: initial_wetdry_node
     type(c_ptr) :: x_cell
     type(c_ptr) :: y_cell
     type(c_ptr) :: h_cell
     type(c_ptr) :: area
     type(c_ptr) :: facenum_at_cell
     type(c_ptr) :: adj_cellnum_at_cell
     type(c_ptr) :: sign_in_outflow
     type(c_ptr) :: bottom_layer_at_element
     type(c_ptr) :: ob_element_flag
     type(c_ptr) :: qb_element_flag
     type(c_ptr) :: x_face
     type(c_ptr) :: y_face
     type(c_ptr) :: h_face
     type(c_ptr) :: face_length
     type(c_ptr) :: delta_j
     type(c_ptr) :: cos_theta
     type(c_ptr) :: sin_theta
     type(c_ptr) :: cos_theta2
     type(c_ptr) :: sin_theta2
     type(c_ptr) :: adj_cellnum_at_face
     type(c_ptr) :: nodenum_at_face
     type(c_ptr) :: bottom_layer_at_face
     type(c_ptr) :: boundary_type_of_face
     type(c_ptr) :: isflowside3
     type(c_ptr) :: ob_cell_id
     type(c_ptr) :: ob_face_id
     type(c_ptr) :: qb_cell
     type(c_ptr) :: qb_face
  end type

  integer(c_int), parameter :: GOM_F_ETA_CELL = 1
  integer(c_int), parameter :: GOM_F_ETA_CELL_NEW = 2
  integer(c_int), parameter :: GOM_F_ETA_NODE = 3
  integer(c_int), parameter :: GOM_F_WETDRY_NODE = 4
  integer(c_int), parameter :: GOM_F_UN_FACE = 5
  integer(c_int), parameter :: GOM_F_VN_FACE = 6
  integer(c_int), parameter :: GOM_F_UN_FACE_NEW = 7
  integer(c_int), parameter :: GOM_F_VN_FACE_NEW = 8
  integer(c_int), parameter :: GOM_F_UN_ELM = 9
  integer(c_int), parameter :: GOM_F_VN_ELM = 10
  integer(c_int), parameter :: GOM_F_WN_CELL = 11
  integer(c_int), parameter :: GOM_F_WN_CELL_NEW = 12
  integer(c_int), parameter :: GOM_F_U_NODE = 13
  integer(c_int), parameter :: GOM_F_V_NODE = 14
  integer(c_int), parameter :: GOM_F_W_NODE = 15
  integer(c_int), parameter :: GOM_F_U_FACE_LEVEL = 16
  integer(c_int), parameter :: GOM_F_V_FACE_LEVEL = 17
  integer(c_int), parameter :: GOM_F_DZ_CELL = 18
  integer(c_int), parameter :: GOM_F_DZ_CELL_NEW = 19
  integer(c_int), parameter :: GOM_F_DZHALF_CELL = 20
  integer(c_int), parameter :: GOM_F_DZHALF_CELL_NEW = 21
  integer(c_int), parameter :: GOM_F_DZ_FACE = 22
  integer(c_int), parameter :: GOM_F_DZ_FACE_NEW = 23
  integer(c_int), parameter :: GOM_F_DZHALF_FACE = 24
  integer(c_int), parameter :: GOM_F_DZHALF_FACE_NEW = 25
  integer(c_int), parameter :: GOM_F_DZ_NODE = 26
  integer(c_int), parameter :: GOM_F_DZ_NODE_NEW = 27
  integer(c_int), parameter :: GOM_F_DZHALF_NODE = 28
  integer(c_int), parameter :: GOM_F_DZHALF_NODE_NEW = 29
  integer(c_int), parameter :: GOM_F_TOP_LAYER_CELL = 30
  integer(c_int), parameter :: GOM_F_TOP_LAYER_FACE = 31
  integer(c_int), parameter :: GOM_F_TOP_LAYER_NODE = 32
  integer(c_int), parameter :: GOM_F_AINVG1 = 33
  integer(c_int), parameter :: GOM_F_AINVG2 = 34
  integer(c_int), parameter :: GOM_F_AINVDZ1 = 35
  integer(c_int), parameter :: GOM_F_AINVDZ2 = 36
  integer(c_int), parameter :: GOM_F_KH = 37
  integer(c_int), parameter :: GOM_F_AV = 38
  integer(c_int), parameter :: GOM_F_KV = 39
  integer(c_int), parameter :: GOM_F_SALT_CELL = 40
  integer(c_int), parameter :: GOM_F_SALT_CELL_NEW = 41
  integer(c_int), parameter :: GOM_F_TEMP_CELL = 42
  integer(c_int), parameter :: GOM_F_TEMP_CELL_NEW = 43
  integer(c_int), parameter :: GOM_F_SALT_NODE = 44
  integer(c_int), parameter :: GOM_F_TEMP_NODE = 45
  integer(c_int), parameter :: GOM_F_SALT_FACE = 46
  integer(c_int), parameter :: GOM_F_TEMP_FACE = 47
  integer(c_int), parameter :: GOM_F_RHO_CELL = 48
  integer(c_int), parameter :: GOM_F_RHO_NODE = 49
  integer(c_int), parameter :: GOM_F_RHO_FACE = 50
  integer(c_int), parameter :: GOM_F_NUM_SUB_ELM = 51
  integer(c_int), parameter :: GOM_F_CDB = 52
  integer(c_int), parameter :: GOM_F_GAMMA_B = 53
  integer(c_int), parameter :: GOM_F_QU_BOUNDARY = 54
  integer(c_int), parameter :: GOM_F_ELM_FOOT = 55
  integer(c_int), parameter :: GOM_F_ELM_NEAR_EDGE = 56
  integer(c_int), parameter :: GOM_F_WIND_STRESS_NORMAL = 57
  integer(c_int), parameter :: GOM_F_WIND_STRESS_TANGNT = 58
  integer(c_int), parameter :: GOM_F_GAMMA_T = 59
  integer(c_int), parameter :: GOM_F_AIR_P = 60
  integer(c_int), parameter :: GOM_F_ETA_AT_OB_OLD = 61
  integer(c_int), parameter :: GOM_F_ETA_AT_OB_NEW = 62
  integer(c_int), parameter :: GOM_F_Q_ADD = 63
  integer(c_int), parameter :: GOM_F_PHI_SW = 64
  integer(c_int), parameter :: GOM_F_PHI_SZ = 65
  integer(c_int), parameter :: GOM_GEO_CONCAVE = 1
  integer(c_int), parameter :: GOM_GEO_AREA = 2
  integer(c_int), parameter :: GOM_GEO_MAX_NB = 3
  integer(c_int), parameter :: GOM_GEO_HANGING = 4
  integer(c_int), parameter :: GOM_GEO_SURROUNDING = 5
  integer(c_int), parameter :: GOM_GEO_FACE_COUNT = 6
  integer(c_int), parameter :: GOM_GEO_FACE_LENGTH = 7
  integer(c_int), parameter :: GOM_GEO_BALL = 8
  integer(c_int), parameter :: GOM_GEO_VORONOI = 9
  integer(c_int), parameter :: GOM_GEO_CENTRES = 10
  integer(c_int), parameter :: GOM_GEO_BOUNDARY = 11
  integer(c_int), parameter :: GOM_GEO_VERTICAL = 12

  interface
     integer(c_int) function gom_abi_version() bind(c, name="gom_abi_version")
       import
     end function
     type(c_ptr) function gom_errstr(code) bind(c, name="gom_errstr")
       import
       integer(c_int), value :: code
     end function
     integer(c_int) function gom_create(dims, params, geom, ctx) bind(c, name="gom_create")
       import
       type(gom_dims), intent(in) :: dims
       type(gom_params), intent(in) :: params
       type(gom_geom), intent(in) :: geom
       type(c_ptr), intent(out) :: ctx
     end function
     subroutine gom_destroy(ctx) bind(c, name="gom_destroy")
       import
       type(c_ptr), value :: ctx
     end subroutine
     integer(c_int) function gom_set_field(ctx, field, host, count) bind(c, name="gom_set_field")
       import
       type(c_ptr), value :: ctx, host
       integer(c_int), value :: field
       integer(c_int64_t), value :: count
     end function
     integer(c_int) function gom_get_field(ctx, field, host, count) bind(c, name="gom_get_field")
       import
       type(c_ptr), value :: ctx, host
       integer(c_int), value :: field
       integer(c_int64_t), value :: count
     end function
     integer(c_int) function gom_set_forcing(ctx, forcing) bind(c, name="gom_set_forcing")
       import
       type(c_ptr), value :: ctx
       type(gom_forcing), intent(in) :: forcing
     end function
     integer(c_int) function gom_step_bottom_friction(ctx) bind(c, name="gom_step_bottom_friction")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_boundary_velocity(ctx) bind(c, name="gom_step_boundary_velocity")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_advection(ctx) bind(c, name="gom_step_advection")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_momentum(ctx) bind(c, name="gom_step_momentum")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_free_surface(ctx, pcg_iters) bind(c, name="gom_step_free_surface")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(out) :: pcg_iters
     end function
     integer(c_int) function gom_step_velocities(ctx) bind(c, name="gom_step_velocities")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_layers(ctx) bind(c, name="gom_step_layers")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_node_velocity(ctx) bind(c, name="gom_step_node_velocity")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_transport(ctx) bind(c, name="gom_step_transport")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_density(ctx) bind(c, name="gom_step_density")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_swap(ctx) bind(c, name="gom_step_swap")
       import
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function gom_step_all(ctx, pcg_iters) bind(c, name="gom_step_all")
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(out) :: pcg_iters
     end function
     integer(c_int) function gom_conservation(ctx, volume, salt_mass) bind(c, name="gom_conservation")
       import
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: volume, salt_mass
     end function
     integer(c_int) function gom_set_boundary_series(ctx, series) bind(c, name="gom_set_boundary_series")
       import
       type(c_ptr), value :: ctx
       type(gom_boundary_series), intent(in) :: series
     end function
     integer(c_int) function gom_push_hurricane_frame(ctx, frame) bind(c, name="gom_push_hurricane_frame")
       import
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: frame(*)
     end function
     integer(c_int) function gom_push_hurricane_center(ctx, x, y, julian_day) bind(c, name="gom_push_hurricane_center")
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: x, y, julian_day
     end function
     integer(c_int) function gom_geometry_build(mesh, out, failure) bind(c, name="gom_geometry_build")
       import
       type(gom_mesh), intent(in) :: mesh
       type(gom_mesh_geometry), intent(inout) :: out
       type(gom_status), intent(out) :: failure
     end function
     integer(c_int) function gom_get_status(ctx, status, clear) bind(c, name="gom_get_status")
       import
       type(c_ptr), value :: ctx
       type(gom_status), intent(out) :: status
       integer(c_int), value :: clear
     end function
  end interface
end module gom_core_abi


module gom_core_shim
  use iso_c_binding
  use gom_core_abi
  use mod_global_variables
  use mod_file_definition, only : pw_run_log
  implicit none
  private
  public :: gom_gpu_init, gom_gpu_step, gom_gpu_get, gom_gpu_set_forcing, gom_gpu_check, gom_ctx, &
       gom_gpu_set_boundary_series

  type(c_ptr), save :: gom_ctx = c_null_ptr
  ! set when the device forms phi_sz / phi_sw itself (gom_gpu_set_boundary_series with the heat
  ! balance): the host's heat_term_by_term result is then not uploaded
  logical, save :: gom_device_heat = .false.
  type(gom_dims), save :: dims
  ! boundary concentrations per transport subcycle, (n, 2, Nt): slot 1 salinity, slot 2 temperature
  real(c_double), allocatable, target, save :: con_ob(:,:,:), con_qb(:,:,:)
  real(c_double), allocatable, target, save :: zeros_f(:)

contains

  ! c_loc of an array's first element (the dummies carry TARGET, so c_loc is allowed; the library
  ! copies during the call)
  type(c_ptr) function cptr_d(a)
    real(c_double), target, intent(in) :: a(*)
    cptr_d = c_loc(a)
  end function
  type(c_ptr) function cptr_i(a)
    integer(c_int32_t), target, intent(in) :: a(*)
    cptr_i = c_loc(a)
  end function

  ! a failed call: print what the device recorded and stop, as the reference's checks do
  subroutine gom_gpu_check(rc, where)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: where
    type(gom_status) :: st
    integer(c_int) :: rc2
    if (rc == GOM_OK) return
    rc2 = gom_get_status(gom_ctx, st, 0_c_int)
    write(pw_run_log,*) 'GPU core failed in ', where, ': code', rc, ' site', st%site, ' entity', st%entity, &
         ' layer', st%layer, ' value', st%value
    write(*,*) 'GPU core failed in ', where, ': code', rc, ' site', st%site, ' entity', st%entity, ' layer', st%layer
    stop
  end subroutine

  ! after prepare_gom (main.f90:47): context from the module arrays, then the state
  subroutine gom_gpu_init()
    type(gom_params) :: p
    type(gom_geom) :: g
    integer(c_int) :: rc
    integer :: nt
    if (gom_abi_version() /= GOM_ABI_VERSION) stop 'libgomcore.so: ABI version mismatch'
    dims = gom_dims(maxele, maxface, maxnod, maxlayer, max_no_neighbor_node, num_ob_cell, num_Qb_cell, 0)
    p%gravity = gravity
    p%rho_o = rho_o
    p%msl = MSL
    p%dt = dt
    p%theta = theta
    p%adv_onoff_depth = adv_onoff_depth
    p%von_karman = von_Karman
    p%cd_const = 0.0_c_double
    p%dry_depth = dry_depth
    p%smagorinsky = Smagorinsky_parameter
    p%ah_0 = Ah_0
    p%kh_0 = Kh_0
    p%error_tolerance = error_tolerance
    p%delta_z_min = delta_z_min
    p%denominator_min_for_matrix = denominator_min_for_matrix
    p%advection_flag = advection_flag
    p%elm_backtrace_flag = ELM_backtrace_flag
    p%elm_sub_iter = ELM_sub_iter
    p%elm_min_iter = ELM_min_iter
    p%elm_max_iter = ELM_max_iter
    p%bf_flag = bf_flag
    p%baroclinic_flag = baroclinic_flag
    p%ana_density = ana_density
    p%max_iteration_pcg = max_iteration_pcg
    p%transport_flag = transport_flag
    p%trans_sub_iter = trans_sub_iter
    p%h_flux_limiter = h_flux_limiter
    p%v_flux_limiter = v_flux_limiter
    p%is_salt = is_salt
    p%is_temp = is_temp
    p%heat_option = heat_option
    p%test_barrier_phantom_blocks = 0
    p%precision = 0
    p%turbulence_flag = 0
    p%transport_solver = transport_solver
    p%pp_h1 = h1_pp
    p%pp_h2 = h2_pp
    p%pp_vdmax1 = vdmax_pp1
    p%pp_vdmax2 = vdmax_pp2
    p%pp_vdmin1 = vdmin_pp1
    p%pp_vdmin2 = vdmin_pp2
    p%pp_tdmin = tdmin_pp
    g%x_node = cptr_d(x_node)
    g%y_node = cptr_d(y_node)
    g%h_node = cptr_d(h_node)
    g%adj_cells_at_node = cptr_i(adj_cells_at_node)
    g%adj_cellnum_at_node = cptr_i(adj_cellnum_at_node)
    g%node_count_each_element = cptr_i(node_count_each_element)
    g%adj_nodes_at_node = cptr_i(adj_nodes_at_node)
    g%adj_nodenum_at_node = cptr_i(adj_nodenum_at_node)
    g%bottom_layer_at_node = cptr_i(bottom_layer_at_node)
    g%initial_wetdry_node = cptr_i(initial_wetdry_node)
    g%x_cell = cptr_d(x_cell)
    g%y_cell = cptr_d(y_cell)
    g%h_cell = cptr_d(h_cell)
    g%area = cptr_d(area)
    g%tri_or_quad = cptr_i(tri_or_quad)
    g%nodenum_at_cell = cptr_i(nodenum_at_cell)
    g%facenum_at_cell = cptr_i(facenum_at_cell)
    g%adj_cellnum_at_cell = cptr_i(adj_cellnum_at_cell)
    g%sign_in_outflow = cptr_i(sign_in_outflow)
    g%bottom_layer_at_element = cptr_i(bottom_layer_at_element(1))   ! declared (0:maxele)
    g%ob_element_flag = cptr_i(ob_element_flag)
    g%qb_element_flag = cptr_i(Qb_element_flag)
    g%x_face = cptr_d(x_face)
    g%y_face = cptr_d(y_face)
    g%h_face = cptr_d(h_face)
    g%face_length = cptr_d(face_length)
    g%delta_j = cptr_d(delta_j)
    g%cos_theta = cptr_d(cos_theta)
    g%sin_theta = cptr_d(sin_theta)
    g%cos_theta2 = cptr_d(cos_theta2)
    g%sin_theta2 = cptr_d(sin_theta2)
    g%adj_cellnum_at_face = cptr_i(adj_cellnum_at_face)
    g%nodenum_at_face = cptr_i(nodenum_at_face)
    g%bottom_layer_at_face = cptr_i(bottom_layer_at_face)
    g%boundary_type_of_face = cptr_i(boundary_type_of_face)
    g%isflowside3 = cptr_i(isflowside3)
    g%coriolis_factor = cptr_d(coriolis_factor)
    g%manning = c_null_ptr
    if (bf_flag == 1) g%manning = cptr_d(manning)
    g%bf_height = c_null_ptr
    if (bf_flag == 2) g%bf_height = cptr_d(bf_height)
    g%ob_cell_id = c_null_ptr
    if (num_ob_cell > 0) g%ob_cell_id = cptr_i(ob_cell_id)
    g%qb_cell = c_null_ptr
    g%qb_face = c_null_ptr
    if (num_Qb_cell > 0) then
       g%qb_cell = cptr_i(Q_boundary(1, 1))
       g%qb_face = cptr_i(Q_boundary(1, 2))
    end if
    g%z_level = cptr_d(z_level)          ! declared (0:maxlayer)
    g%delta_z = cptr_d(delta_z)
    g%run_cell_start = c_null_ptr
    g%run_face_start = c_null_ptr
    g%run_node_start = c_null_ptr
    g%run_ob_start = c_null_ptr
    rc = gom_create(dims, p, g, gom_ctx)
    call gom_gpu_check(rc, 'gom_create')
    nt = max(trans_sub_iter, 1)
    allocate(con_ob(max(num_ob_cell, 1), 2, nt), con_qb(max(num_Qb_cell, 1), 2, nt), zeros_f(maxface))
    con_ob = 0.0_c_double
    con_qb = 0.0_c_double
    zeros_f = 0.0_c_double
    ! the state prepare_gom left (cold or hot start)
    call put_d(GOM_F_ETA_CELL, eta_cell, size(eta_cell))
    call put_d(GOM_F_ETA_CELL_NEW, eta_cell_new, size(eta_cell_new))
    call put_d(GOM_F_ETA_NODE, eta_node, size(eta_node))
    call put_i(GOM_F_WETDRY_NODE, wetdry_node, size(wetdry_node))
    call put_d(GOM_F_UN_FACE, un_face, size(un_face))
    call put_d(GOM_F_VN_FACE, vn_face, size(vn_face))
    call put_d(GOM_F_UN_FACE_NEW, un_face_new, size(un_face_new))
    call put_d(GOM_F_VN_FACE_NEW, vn_face_new, size(vn_face_new))
    call put_d(GOM_F_UN_ELM, un_ELM, size(un_ELM))
    call put_d(GOM_F_VN_ELM, vn_ELM, size(vn_ELM))
    call put_d(GOM_F_WN_CELL, wn_cell, size(wn_cell))
    call put_d(GOM_F_WN_CELL_NEW, wn_cell_new, size(wn_cell_new))
    call put_d(GOM_F_U_NODE, u_node, size(u_node))
    call put_d(GOM_F_V_NODE, v_node, size(v_node))
    call put_d(GOM_F_W_NODE, w_node, size(w_node))
    call put_d(GOM_F_U_FACE_LEVEL, u_face_level, size(u_face_level))
    call put_d(GOM_F_V_FACE_LEVEL, v_face_level, size(v_face_level))
    call put_d(GOM_F_DZ_CELL, dz_cell, size(dz_cell))
    call put_d(GOM_F_DZ_CELL_NEW, dz_cell_new, size(dz_cell_new))
    call put_d(GOM_F_DZHALF_CELL, dzhalf_cell, size(dzhalf_cell))
    call put_d(GOM_F_DZHALF_CELL_NEW, dzhalf_cell_new, size(dzhalf_cell_new))
    call put_d(GOM_F_DZ_FACE, dz_face, size(dz_face))
    call put_d(GOM_F_DZ_FACE_NEW, dz_face_new, size(dz_face_new))
    call put_d(GOM_F_DZHALF_FACE, dzhalf_face, size(dzhalf_face))
    call put_d(GOM_F_DZHALF_FACE_NEW, dzhalf_face_new, size(dzhalf_face_new))
    call put_d(GOM_F_DZ_NODE, dz_node, size(dz_node))
    call put_d(GOM_F_DZ_NODE_NEW, dz_node_new, size(dz_node_new))
    call put_d(GOM_F_DZHALF_NODE, dzhalf_node, size(dzhalf_node))
    call put_d(GOM_F_DZHALF_NODE_NEW, dzhalf_node_new, size(dzhalf_node_new))
    call put_i(GOM_F_TOP_LAYER_CELL, top_layer_at_element(1), maxele)
    call put_i(GOM_F_TOP_LAYER_FACE, top_layer_at_face, size(top_layer_at_face))
    call put_i(GOM_F_TOP_LAYER_NODE, top_layer_at_node, size(top_layer_at_node))
    call put_d(GOM_F_KH, Kh, size(Kh))
    call put_d(GOM_F_AV, Av, size(Av))
    call put_d(GOM_F_KV, Kv, size(Kv))
    call put_d(GOM_F_SALT_CELL, salt_cell, size(salt_cell))
    call put_d(GOM_F_SALT_CELL_NEW, salt_cell_new, size(salt_cell_new))
    call put_d(GOM_F_TEMP_CELL, temp_cell, size(temp_cell))
    call put_d(GOM_F_TEMP_CELL_NEW, temp_cell_new, size(temp_cell_new))
    call put_d(GOM_F_SALT_NODE, salt_node, size(salt_node))
    call put_d(GOM_F_TEMP_NODE, temp_node, size(temp_node))
    call put_d(GOM_F_SALT_FACE, salt_face, size(salt_face))
    call put_d(GOM_F_TEMP_FACE, temp_face, size(temp_face))
    call put_d(GOM_F_RHO_CELL, rho_cell, size(rho_cell))
    call put_d(GOM_F_RHO_NODE, rho_node, size(rho_node))
    call put_d(GOM_F_RHO_FACE, rho_face, size(rho_face))
    call put_i(GOM_F_NUM_SUB_ELM, num_sub_elm_iteration, size(num_sub_elm_iteration))
  end subroutine

  ! upload n elements of a module array (its whole size) as a state field
  subroutine put_d(field, a, n)
    integer(c_int), intent(in) :: field
    real(c_double), target, intent(in) :: a(*)
    integer, intent(in) :: n
    call gom_gpu_check(gom_set_field(gom_ctx, field, c_loc(a), int(n, c_int64_t)), 'gom_set_field')
  end subroutine
  subroutine put_i(field, a, n)
    integer(c_int), intent(in) :: field
    integer(c_int32_t), target, intent(in) :: a(*)
    integer, intent(in) :: n
    call gom_gpu_check(gom_set_field(gom_ctx, field, c_loc(a), int(n, c_int64_t)), 'gom_set_field')
  end subroutine

  ! a field back into its module array (output writers, restart, termination checks):
  ! call gom_gpu_get(GOM_F_SALT_CELL, salt_cell, size(salt_cell))
  subroutine gom_gpu_get(field, a, n)
    integer(c_int), intent(in) :: field
    real(c_double), target, intent(inout) :: a(*)
    integer, intent(in) :: n
    call gom_gpu_check(gom_get_field(gom_ctx, field, c_loc(a), int(n, c_int64_t)), 'gom_get_field')
  end subroutine

  ! the host forcing of this step (main.f90:85-161 computed it into the module arrays) and the
  ! boundary concentrations of every transport subcycle (solve_transport_equation_v19.f90:229-397)
  subroutine gom_gpu_set_forcing()
    type(gom_forcing) :: f
    integer :: s, nt, i
    real(dp) :: dt2, u2
    nt = max(trans_sub_iter, 1)
    dt2 = dt / nt
    do s = 0, nt - 1
       u2 = (julian_day*86400.0 - dt) + (s + 1)*dt2
       do i = 1, num_ob_cell
          if (is_salt == 1 .and. salt_ser_id(i) > 0) con_ob(i, 1, s + 1) = spinup_function_baroclinic * &
               series_at(salt_ser_time(:, salt_ser_id(i)), salt_ser_salt(:, salt_ser_id(i)), &
               salt_ser_data_num(salt_ser_id(i)), u2)
          if (is_temp == 1 .and. temp_ser_id(i) > 0) con_ob(i, 2, s + 1) = spinup_function_baroclinic * &
               series_at(temp_ser_time(:, temp_ser_id(i)), temp_ser_temp(:, temp_ser_id(i)), &
               temp_ser_data_num(temp_ser_id(i)), u2)
       end do
       do i = 1, num_Qb_cell
          if (is_salt == 1 .and. Q_salt_ser_id(i) > 0) con_qb(i, 1, s + 1) = spinup_function_baroclinic * &
               series_at(salt_ser_time(:, Q_salt_ser_id(i)), salt_ser_salt(:, Q_salt_ser_id(i)), &
               salt_ser_data_num(Q_salt_ser_id(i)), u2)
          if (is_temp == 1 .and. Q_temp_ser_id(i) > 0) con_qb(i, 2, s + 1) = spinup_function_baroclinic * &
               series_at(temp_ser_time(:, Q_temp_ser_id(i)), temp_ser_temp(:, Q_temp_ser_id(i)), &
               temp_ser_data_num(Q_temp_ser_id(i)), u2)
       end do
    end do
    f%elapsed_time = elapsed_time
    f%spinup_tide = spinup_function_tide
    f%spinup_baroclinic = spinup_function_baroclinic
    f%reserved = 0.0_c_double
    f%eta_at_ob_old = c_null_ptr
    f%eta_at_ob_new = c_null_ptr
    if (num_ob_cell > 0) then
       f%eta_at_ob_old = cptr_d(eta_at_ob_old)
       f%eta_at_ob_new = cptr_d(eta_at_ob_new)
    end if
    f%q_add = c_null_ptr
    if (num_Qb_cell > 0) f%q_add = cptr_d(Q_add)
    f%wind_stress_normal = cptr_d(wind_stress_normal)
    f%wind_stress_tangnt = cptr_d(wind_stress_tangnt)
    f%gamma_t = cptr_d(Gamma_T)
    f%air_p = cptr_d(air_p1)
    f%con_at_ob = cptr_d(con_ob)
    f%con_at_qb = cptr_d(con_qb)
    f%phi_sw = c_null_ptr
    f%phi_sz = c_null_ptr
    if (is_temp == 1 .and. heat_option == 2) f%phi_sw = cptr_d(phi_sw)
    if (is_temp == 1 .and. heat_option == 1 .and. .not. gom_device_heat) f%phi_sz = cptr_d(phi_sz)
    call gom_gpu_check(gom_set_forcing(gom_ctx, f), 'gom_set_forcing')
  end subroutine

  ! The boundary tables of mod_global_variables held on the device (gom_set_boundary_series): the
  ! harmonic constituents (read_harmonic_ser.f90), the elevation, discharge, salinity and
  ! temperature series (read_eta_ser.f90, read_q_ser.f90, read_salt_ser.f90, read_temp_ser.f90) and
  ! the ids of cards C20_1 / C22_1.  Call once after prepare_gom (step 0) or after a hot start (the
  ! step it restarts from); every later gom_gpu_step then advances the clock and forms
  ! setup_spinup, compute_boundary_eta, calculate_Q and the boundary concentrations of every
  ! subcycle on the device.  With station wind (wind_flag 1, heat_model_flag 0, card C30) the
  ! device also forms get_windp_at_face and calculate_wind_stress every step, so
  ! gom_gpu_set_forcing is then needed only for the heat terms.
  subroutine gom_gpu_set_boundary_series(step)
    integer, intent(in) :: step
    type(gom_boundary_series) :: bs
    integer(c_int32_t), allocatable, target, save :: se(:), sq(:), ss(:), st(:), hs(:)
    real(c_double), allocatable, target, save :: te(:), ve(:), tq(:), vq(:), ts(:), vs(:), tt(:), vt(:)
    real(c_double), allocatable, target, save :: amp(:), per(:), nod(:), eq(:), ph(:), shift(:), portion(:)
    integer(c_int32_t), allocatable, target, save :: obt(:), obh(:), obe(:), obs(:), obtm(:), qq(:), qs(:), qt(:)
    integer(c_int32_t), allocatable, target, save :: swu(:), swv(:), wnode(:)
    real(c_double), allocatable, target, save :: hframes(:), airt(:), airv(:)
    real(c_double), allocatable, target, save :: twu(:), vwu(:), twv(:), vwv(:)
    integer :: h, j, m, nc
    ! a kind without series (its reader's arrays unallocated) is passed as n_series = 0
    bs%eta = gom_series(0, 0, c_null_ptr, c_null_ptr, c_null_ptr)
    bs%q = bs%eta
    bs%salt = bs%eta
    bs%temp = bs%eta
    bs%wind_u = bs%eta
    bs%wind_v = bs%eta
    if (num_eta_ser > 0) call pack_series(num_eta_ser, eta_ser_data_num, eta_ser_time, eta_ser_eta, se, te, ve, bs%eta)
    if (num_Q_ser > 0) call pack_series(num_Q_ser, q_data_num, q_ser_time, q_ser_Q, sq, tq, vq, bs%q)
    if (is_salt == 1 .and. num_salt_ser > 0) &
         call pack_series(num_salt_ser, salt_ser_data_num, salt_ser_time, salt_ser_salt, ss, ts, vs, bs%salt)
    if (is_temp == 1 .and. num_temp_ser > 0) &
         call pack_series(num_temp_ser, temp_ser_data_num, temp_ser_time, temp_ser_temp, st, tt, vt, bs%temp)
    ! harmonic series: constituents one series after another, offsets in hs
    if (allocated(hs)) deallocate(hs, amp, per, nod, eq, ph, shift)
    nc = 0
    do h = 1, num_harmonic_ser
       nc = nc + no_tidal_constituent(h)
    end do
    allocate(hs(num_harmonic_ser + 1), amp(max(nc, 1)), per(max(nc, 1)), nod(max(nc, 1)), eq(max(nc, 1)), &
         ph(max(nc, 1)), shift(max(num_harmonic_ser, 1)))
    hs(1) = 0
    m = 0
    do h = 1, num_harmonic_ser
       do j = 1, no_tidal_constituent(h)
          m = m + 1
          amp(m) = tidal_amplitude(j, h)
          per(m) = tidal_period(j, h)
          nod(m) = tidal_nodal_factor(j, h)
          eq(m) = equilibrium_argument(j, h)
          ph(m) = tidal_phase(j, h)
       end do
       shift(h) = tidal_phase_shift(h)
       hs(h + 1) = m
    end do
    if (allocated(obt)) deallocate(obt, obh, obe, obs, obtm, qq, qs, qt, portion)
    allocate(obt(max(num_ob_cell, 1)), obh(max(num_ob_cell, 1)), obe(max(num_ob_cell, 1)), &
         obs(max(num_ob_cell, 1)), obtm(max(num_ob_cell, 1)), qq(max(num_Qb_cell, 1)), qs(max(num_Qb_cell, 1)), &
         qt(max(num_Qb_cell, 1)), portion(max(num_Qb_cell, 1)))
    do j = 1, num_ob_cell
       obt(j) = ob_eta_type(j)
       obh(j) = harmonic_ser_id(j)
       obe(j) = eta_ser_id(j)
       obs(j) = salt_ser_id(j)
       obtm(j) = temp_ser_id(j)
    end do
    do j = 1, num_Qb_cell
       qq(j) = Q_ser_id(j)
       qs(j) = Q_salt_ser_id(j)
       qt(j) = Q_temp_ser_id(j)
       portion(j) = Q_portion(j)
    end do
    bs%julian_day = julian_day
    bs%tide_spinup_period = tide_spinup_period
    bs%baroclinic_spinup_period = baroclinic_spinup_period
    bs%step = step
    bs%reference_diff_days = reference_diff_days
    bs%tide_spinup = tide_spinup
    bs%baroclinic_spinup = baroclinic_spinup
    bs%q_interp_method = q_interp_method
    bs%n_harmonic = num_harmonic_ser
    bs%ob_eta_type = cptr_i(obt)
    bs%ob_harmonic_id = cptr_i(obh)
    bs%ob_eta_id = cptr_i(obe)
    bs%ob_salt_id = cptr_i(obs)
    bs%ob_temp_id = cptr_i(obtm)
    bs%qb_q_id = cptr_i(qq)
    bs%qb_salt_id = cptr_i(qs)
    bs%qb_temp_id = cptr_i(qt)
    bs%qb_portion = cptr_d(portion)
    bs%harmonic_start = cptr_i(hs)
    bs%amplitude = cptr_d(amp)
    bs%period_h = cptr_d(per)
    bs%nodal = cptr_d(nod)
    bs%eq_arg = cptr_d(eq)
    bs%phase = cptr_d(ph)
    bs%phase_shift = cptr_d(shift)
    ! station wind: both components share windp_ser_time
    bs%wind_flag = 0
    bs%wind_formular = wind_formular
    bs%wind_spinup = wind_spinup
    bs%n_wind = 0
    bs%wind_spinup_period = wind_spinup_period
    bs%rho_a = rho_a
    bs%wind_station_node = c_null_ptr
    if (wind_flag == 1 .and. heat_model_flag == 0 .and. num_windp_ser > 0) then
       bs%wind_flag = 1
       bs%n_wind = num_windp_ser
       call pack_series(num_windp_ser, windp_ser_data_num, windp_ser_time, windp_u, swu, twu, vwu, bs%wind_u)
       call pack_series(num_windp_ser, windp_ser_data_num, windp_ser_time, windp_v, swv, twv, vwv, bs%wind_v)
       if (allocated(wnode)) deallocate(wnode)
       allocate(wnode(num_windp_ser))
       if (num_windp_ser > 1) then
          do j = 1, num_windp_ser
             wnode(j) = windp_station_node(j)
          end do
          bs%wind_station_node = cptr_i(wnode)
       end if
    end if
    ! hurricane node frames (card C31, method 1): wind_u0 / v0 / air_p0, wind_u1 .., wind_u2 ..
    bs%hurricane_flag = 0
    bs%hurricane_read_interval = 1
    bs%hurricane_start_jday = 0.0_dp
    bs%hurricane_end_jday = 0.0_dp
    bs%hurricane_frames = c_null_ptr
    bs%hurricane_interp_method = 1
    bs%reserved_hurricane = 0
    bs%hurricane_track = 0.0_dp
    if (hurricane_flag == 1 .and. (hurricane_interp_method == 1 .or. hurricane_interp_method == 2)) then
       if (allocated(hframes)) deallocate(hframes)
       allocate(hframes(9 * maxnod))
       hframes(1:maxnod) = wind_u0
       hframes(maxnod + 1:2 * maxnod) = wind_v0
       hframes(2 * maxnod + 1:3 * maxnod) = air_p0
       hframes(3 * maxnod + 1:4 * maxnod) = wind_u1
       hframes(4 * maxnod + 1:5 * maxnod) = wind_v1
       hframes(5 * maxnod + 1:6 * maxnod) = air_p1
       hframes(6 * maxnod + 1:7 * maxnod) = wind_u2
       hframes(7 * maxnod + 1:8 * maxnod) = wind_v2
       hframes(8 * maxnod + 1:9 * maxnod) = air_p2
       bs%hurricane_flag = 1
       bs%hurricane_read_interval = hurricane_read_interval
       bs%hurricane_start_jday = hurricane_start_jday
       bs%hurricane_end_jday = hurricane_end_jday
       bs%hurricane_frames = cptr_d(hframes)
       bs%hurricane_interp_method = hurricane_interp_method
       if (hurricane_interp_method == 2) then
          ! read_hurricane_ser_0.f90:58-82: the two centres read so far
          bs%hurricane_track = (/ hurric_x_1, hurric_y_1, hurricane_time_1, hurric_x_2, hurric_y_2, &
               hurricane_time_2 /)
       end if
    end if
    ! heat balance (card C7_3 / C7_4, air_ser.inp): heat_term_by_term with sol_swr 2 on the device
    bs%heat_flag = 0
    bs%sol_swr = sol_swr
    bs%n_air = 0
    bs%reserved_heat = 0
    bs%fwz_a = fWz_a
    bs%fwz_b = fWz_b
    bs%fwz_c = fWz_c
    bs%wind_height = wind_height
    bs%light_extinction = light_extinction
    bs%sol_absorb = sol_absorb
    bs%sed_water_exchange = sed_water_exchange
    bs%t_sed = T_sed
    bs%sed_temp_coeff = sed_temp_coeff
    bs%air_time = c_null_ptr
    bs%air_values = c_null_ptr
    bs%year = year
    bs%month = month
    bs%lon = lon
    bs%lat = lat
    gom_device_heat = .false.
    if (transport_flag == 1 .and. is_temp == 1 .and. heat_option == 1 .and. (sol_swr == 1 .or. sol_swr == 2)) then
       if (allocated(airt)) deallocate(airt, airv)
       allocate(airt(max(max_air_data_num, 1)), airv(5 * max(max_air_data_num, 1)))
       do j = 1, max_air_data_num
          airt(j) = air_ser_time(j)
          airv(j) = T_air(j)
          airv(max_air_data_num + j) = T_dew(j)
          airv(2 * max_air_data_num + j) = air_wind_speed(j)
          airv(3 * max_air_data_num + j) = solar_radiation(j)
          airv(4 * max_air_data_num + j) = cloud(j)
       end do
       bs%heat_flag = 1
       bs%n_air = max_air_data_num
       bs%air_time = cptr_d(airt)
       bs%air_values = cptr_d(airv)
       gom_device_heat = .true.
    end if
    call gom_gpu_check(gom_set_boundary_series(gom_ctx, bs), 'gom_set_boundary_series')
  end subroutine

  ! one kind of series, (max_len, n) columns with their lengths, as concatenated samples with offsets
  subroutine pack_series(n, counts, times, values, start, t, v, ser)
    integer, intent(in) :: n
    integer, intent(in) :: counts(:)
    real(dp), intent(in) :: times(:, :), values(:, :)
    integer(c_int32_t), allocatable, target, intent(inout) :: start(:)
    real(c_double), allocatable, target, intent(inout) :: t(:), v(:)
    type(gom_series), intent(out) :: ser
    integer :: k, q, m
    if (allocated(start)) deallocate(start, t, v)
    m = 0
    do k = 1, n
       m = m + counts(k)
    end do
    allocate(start(n + 1), t(max(m, 1)), v(max(m, 1)))
    start(1) = 0
    m = 0
    do k = 1, n
       do q = 1, counts(k)
          m = m + 1
          t(m) = times(q, k)
          v(m) = values(q, k)
       end do
       start(k + 1) = m
    end do
    ser%n_series = n
    ser%reserved = 0
    ser%start = cptr_i(start)
    ser%time = cptr_d(t)
    ser%value = cptr_d(v)
  end subroutine

  ! linear interpolation of a series at model time u2 (series time minus reference_diff_days)
  real(dp) function series_at(t, v, n, u2)
    real(dp), intent(in) :: t(:), v(:), u2
    integer, intent(in) :: n
    integer :: t2
    real(dp) :: u1, u3
    series_at = 0.0_dp
    do t2 = 2, n
       u1 = t(t2 - 1) - reference_diff_days * 86400.0
       u3 = t(t2) - reference_diff_days * 86400.0
       if (u2 >= u1 .and. u2 <= u3) then
          series_at = (u2 - u1)*(v(t2) - v(t2 - 1))/(u3 - u1) + v(t2 - 1)
          exit
       end if
    end do
  end function

  ! main.f90:167-272 as one captured graph, after the host forcing of main.f90:85-161
  subroutine gom_gpu_step()
    integer(c_int32_t) :: iters
    call gom_gpu_set_forcing()
    call gom_gpu_check(gom_step_all(gom_ctx, iters), 'gom_step_all')
  end subroutine
end module gom_core_shim


! ------------------------------------------------------------------------------------------------
! The time loop's subroutines, same names, forwarding to the core.  The state stays on the GPU
! between them; the output writers call gom_gpu_get for what they write.
subroutine calculate_bottom_friction
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_bottom_friction(gom_ctx), 'calculate_bottom_friction')
end subroutine

subroutine gom_boundary_velocity
  ! replaces the core part of compute_boundary_velocity.f90 (after its host call of calculate_Q)
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_set_forcing()
  call gom_gpu_check(gom_step_boundary_velocity(gom_ctx), 'compute_boundary_velocity')
end subroutine

subroutine solve_nonlinear_advection
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_set_forcing()        ! compute_boundary_eta ran on the host just before
  call gom_gpu_check(gom_step_advection(gom_ctx), 'solve_nonlinear_advection')
end subroutine

subroutine solve_momentum_equation
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_momentum(gom_ctx), 'solve_momentum_equation')
end subroutine

subroutine solve_free_surface_equation
  use iso_c_binding
  use gom_core_shim
  use gom_core_abi
  integer(c_int32_t) :: iters
  call gom_gpu_check(gom_step_free_surface(gom_ctx, iters), 'solve_free_surface_equation')
end subroutine

subroutine solve_velocities
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_velocities(gom_ctx), 'solve_velocities')
end subroutine

subroutine update_vertical_layers_1
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_layers(gom_ctx), 'update_vertical_layers_1')
end subroutine

subroutine calculate_velocity_at_node
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_node_velocity(gom_ctx), 'calculate_velocity_at_node')
end subroutine

subroutine solve_transport_equation_v19
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_set_forcing()        ! heat terms and boundary series of this step
  call gom_gpu_check(gom_step_transport(gom_ctx), 'solve_transport_equation_v19')
end subroutine

subroutine calculate_density_full
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_density(gom_ctx), 'calculate_density_full')
end subroutine

subroutine calculate_density_linear
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_density(gom_ctx), 'calculate_density_linear')
end subroutine

subroutine update_variables
  use gom_core_shim
  use gom_core_abi
  call gom_gpu_check(gom_step_swap(gom_ctx), 'update_variables')
end subroutine

subroutine read_hurricane_ser_1
  ! With the boundary series on the device (gom_gpu_set_boundary_series) the ramp, the face winds,
  ! air_p1 and the drag law run there; on a read step this replacement only reads the next record
  ! of hurricane_ser.inp (read_hurricane_ser_1.f90:34-46) and hands it to the device, which takes it
  ! in this step.
  use iso_c_binding
  use gom_core_shim
  use gom_core_abi
  use mod_global_variables
  use mod_file_definition
  real(c_double), allocatable :: rec(:)
  integer :: i, j
  if (mod(it, hurricane_read_interval) /= 0) return
  allocate(rec(3 * maxnod))
  do i = 1, maxnod
     if (hurricane_data_type == 1) then
        read(pw_hurricane_ser, *) j, rec(i), rec(maxnod + i), rec(2 * maxnod + i)
     else
        read(pw_hurricane_ser) j, rec(i), rec(maxnod + i), rec(2 * maxnod + i)
     end if
     rec(2 * maxnod + i) = rec(2 * maxnod + i) * 100.0_dp
  end do
  call gom_gpu_check(gom_push_hurricane_frame(gom_ctx, rec), 'read_hurricane_ser_1')
  deallocate(rec)
end subroutine

subroutine read_hurricane_ser_2
  ! Method 2: the device moves the frames with the storm centre (IDW_5 over the neighbour lists it
  ! built); on a read step this replacement only reads the next centre record and the next frame
  ! (read_hurricane_ser_2.f90:38-60) and hands both to the device, which takes them in this step.
  use iso_c_binding
  use gom_core_shim
  use gom_core_abi
  use mod_global_variables
  use mod_file_definition
  real(c_double), allocatable :: rec(:)
  integer :: i, j
  if (mod(it, hurricane_read_interval) /= 0) return
  read(pw_hurricane_center, *) hurric_year_2, hurric_month_2, hurric_day_2, hurric_hour_2, hurric_minute_2, &
       hurric_x_2, hurric_y_2, hurric_latitude_2, hurric_delta_pressure_2, hurric_mwr_2
  call julian(hurric_year_2, hurric_month_2, hurric_day_2, hurric_hour_2, hurric_minute_2, 0, &
       hurric_julian_day_2, hurric_julian_day_1900_2)
  call gom_gpu_check(gom_push_hurricane_center(gom_ctx, hurric_x_2, hurric_y_2, hurric_julian_day_2), &
       'read_hurricane_ser_2')
  allocate(rec(3 * maxnod))
  do i = 1, maxnod
     if (hurricane_data_type == 1) then
        read(pw_hurricane_ser, *) j, rec(i), rec(maxnod + i), rec(2 * maxnod + i)
     else
        read(pw_hurricane_ser) j, rec(i), rec(maxnod + i), rec(2 * maxnod + i)
     end if
     rec(2 * maxnod + i) = rec(2 * maxnod + i) * 100.0_dp
  end do
  call gom_gpu_check(gom_push_hurricane_frame(gom_ctx, rec), 'read_hurricane_ser_2')
  deallocate(rec)
end subroutine
