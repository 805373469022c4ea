/*
 * gom_core.h -- C ABI of the GB300 per-timestep core of the General Ocean Model (GOM).
 *
 * GOM's Fortran driver (GOM_Rv1.1.0/source/main.f90) calls its per-timestep subroutines
 * without arguments; they exchange data through module globals declared in
 * GOM_Rv1.1.0/source/mod_global_variables.f90 and allocated in allocate_variables.f90.
 * This header replaces those calls with explicit entry points that take plain pointers
 * and sizes.  Two libraries export exactly these symbols:
 *
 *   libgomcore.so    -- the product: hand-written CUDA for sm_103a, state resident in HBM;
 *   libgomoracle.so  -- a serial FP64 CPU restatement used only as the test checker.
 *
 * Array conventions (identical to the Fortran module arrays, so a Fortran caller passes
 * c_loc() of its arrays unchanged):
 *   - column-major "(k, entity)" storage: layer index fastest, entity slowest;
 *   - an array declared (lo:hi, N) in Fortran has (hi-lo+1)*N elements and element
 *     (k, e) (k in lo..hi, e in 1..N) lives at offset (e-1)*(hi-lo+1) + (k-lo);
 *   - connectivity is 1-based with 0 meaning "none";
 *   - real(dp) is double, integer is int32_t.
 *
 * Error model: every call returns GOM_OK (0) or a positive gom_err code.  Conditions on
 * which the reference executes `stop` are reported as codes; the library never aborts
 * the process.  gom_get_status() returns the first failing site, entity and layer.
 *
 * Threading: a context is not re-entrant.  All device work of a context runs on one
 * CUDA stream owned by the context.  Host arrays are only read during a call.
 */
#ifndef GOM_CORE_H
#define GOM_CORE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GOM_ABI_VERSION 4

typedef struct gom_ctx gom_ctx;

/* ------------------------------------------------------------------ error codes */
typedef enum gom_err {
    GOM_OK = 0,
    GOM_E_ARG = 1,            /* bad argument, size mismatch, unsupported option            */
    GOM_E_CUDA = 2,           /* CUDA runtime error (message via gom_last_message)          */
    GOM_E_NOT_SPD = 3,        /* solve_free_surface_equation.f90:100-104                    */
    GOM_E_ZERO_PIVOT = 4,     /* tridiagonal_solver.f90:32-35,47-50                         */
    GOM_E_ELM = 5,            /* ELM geometry failure: search_straight_line.f90,
                                 ELM_backtrace_v1.f90, bilinear_interpolation.f90 stops     */
    GOM_E_DRY = 6,            /* wet element with dry nodes/sides, dry river boundary       */
    GOM_E_LAYER = 7,          /* impossible elevation/layer: update_vertical_layers_1.f90   */
    GOM_E_DENSITY = 8,        /* calculate_density_full.f90:43-53,103-107                   */
    GOM_E_PCG_MAXIT = 9,      /* warning: PCG hit max_iteration_pcg (the reference goes on) */
    GOM_E_TIMEOUT = 10,       /* a bounded device-side wait gave up                         */
    GOM_E_NOMEM = 11          /* device allocation failed                                   */
} gom_err;

/* Sub-sites recorded in gom_status.site for GOM_E_ELM, one per reference `stop`. */
enum {
    GOM_ELM_START_DRY = 1,        /* search_straight_line.f90:37-46   */
    GOM_ELM_START_OUTSIDE = 2,    /* search_straight_line.f90:82-89   */
    GOM_ELM_ZERO_PATH = 3,        /* search_straight_line.f90:129-139 */
    GOM_ELM_NO_FIRST_EDGE = 4,    /* search_straight_line.f90:162-169 */
    GOM_ELM_OVERSHOOT = 5,        /* search_straight_line.f90:199-207 */
    GOM_ELM_ZERO_REMAIN = 6,      /* search_straight_line.f90:218-222 */
    GOM_ELM_FACE_MISMATCH = 7,    /* search_straight_line.f90:237-242 */
    GOM_ELM_NO_NEXT_EDGE = 8,     /* search_straight_line.f90:343-353 */
    GOM_ELM_END_DRY = 9,          /* search_straight_line.f90:363-372 */
    GOM_ELM_Z_RANGE = 10,         /* search_straight_line.f90:379-385 */
    GOM_ELM_Z_ABOVE = 11,         /* ELM_backtrace_v1.f90:107-113     */
    GOM_ELM_QUAD_OUTSIDE = 12,    /* ELM_backtrace_v1.f90:164-170     */
    GOM_ELM_BILINEAR = 13,        /* bilinear_interpolation.f90:41-113 */
    GOM_ELM_ALL_DRY = 14,         /* ELM_backtrace_v1.f90:275-277 (ELM transport) */
    GOM_ELM_NEG_SUBELEMENT = 15,  /* ELM_backtrace_v1.f90:420-423 (ELM transport) */
    GOM_ELM_NO_SUBELEMENT = 16    /* ELM_backtrace_v1.f90:463-467 (ELM transport) */
};

/* Kind of entity gom_status.entity indexes. */
enum {
    GOM_ENTITY_OTHER = 0,         /* a boundary index, a solver block, or none */
    GOM_ENTITY_CELL = 1,
    GOM_ENTITY_FACE = 2,
    GOM_ENTITY_NODE = 3
};

typedef struct gom_status {
    int32_t code;        /* gom_err of the first failure, 0 if none            */
    int32_t site;        /* sub-site (GOM_ELM_*) or reference line of the stop */
    int32_t entity;      /* 1-based face / cell / node index                   */
    int32_t layer;       /* layer index, 0 if not applicable                    */
    double value;        /* offending value where the reference prints one     */
    int32_t entity_kind; /* GOM_ENTITY_* of entity (no reference counterpart)  */
    int32_t run;         /* packed context: 0-based run holding the entity, found from the
                            run_*_start tables (0 in a single-run context); -1 when the entity is
                            not a cell, face or node (no reference counterpart) */
} gom_status;

/* ------------------------------------------------------------------ sizes */
typedef struct gom_dims {
    int32_t n_cells;    /* maxele                  */
    int32_t n_faces;    /* maxface                 */
    int32_t n_nodes;    /* maxnod                  */
    int32_t n_layers;   /* maxlayer                */
    int32_t max_nb;     /* max_no_neighbor_node    */
    int32_t n_ob;       /* num_ob_cell             */
    int32_t n_qb;       /* num_Qb_cell             */
    int32_t n_runs;     /* independent runs packed into this context (0 or 1: one run; no
                           reference counterpart).  A packed context holds several runs' meshes
                           as one disconnected mesh: each run's cells, faces, nodes and open-
                           boundary cells are contiguous, connectivity is global, and every
                           phase advances all runs in one launch; the free-surface solve keeps a
                           separate PCG (own scalars, own stop test) per run. */
} gom_dims;

/* ------------------------------------------------------------------ scalar configuration
 * Card numbers refer to main.inp as parsed by read_main_inp.f90. */
typedef struct gom_params {
    double gravity;            /* C01 */
    double rho_o;              /* C01 */
    double msl;                /* C2  MSL */
    double dt;                 /* C3  */
    double theta;              /* C5_01 */
    double adv_onoff_depth;    /* C5_01 */
    double von_karman;         /* C5_02 */
    double cd_const;           /* bf_flag == 3 only: constant drag coefficient (extension) */
    double dry_depth;          /* C5_03 */
    double smagorinsky;        /* C5_04 Smagorinsky_parameter */
    double ah_0;               /* C5_04 */
    double kh_0;               /* C5_04 */
    double error_tolerance;    /* C6 */
    double delta_z_min;        /* derived in read_main_inp.f90 card C2_1 */
    double denominator_min_for_matrix; /* derived in read_main_inp.f90 card C5_03 */
    int32_t advection_flag;    /* C5_01 */
    int32_t elm_backtrace_flag;/* C5_01 */
    int32_t elm_sub_iter;      /* C5_01 */
    int32_t elm_min_iter;      /* C5_01 */
    int32_t elm_max_iter;      /* C5_01 */
    int32_t bf_flag;           /* C5_02: 0 none, 1 Manning, 2 log law, 3 constant Cd (extension) */
    int32_t baroclinic_flag;   /* C5_03 */
    int32_t ana_density;       /* C5_03: 0 full UNESCO EOS, 1 linear */
    int32_t max_iteration_pcg; /* C6 */
    int32_t transport_flag;    /* C7 */
    int32_t trans_sub_iter;    /* C7_1 */
    int32_t h_flux_limiter;    /* C7_1 */
    int32_t v_flux_limiter;    /* C7_1 */
    int32_t is_salt;           /* C7_2 is_tran(1) */
    int32_t is_temp;           /* C7_2 is_tran(2) */
    int32_t heat_option;       /* C7_3: 1 per-layer source phi_sz, 2 surface term phi_sw (both
                                  arrays come with gom_set_forcing; their heat-balance models stay
                                  with the host) */
    int32_t test_barrier_phantom_blocks; /* tests only, normally 0: grid barriers of the PCG wait for
                                            this many blocks that do not exist, so their bounded wait
                                            runs out and the solve reports GOM_E_TIMEOUT */
    int32_t precision;         /* GOM_PRECISION_FP64 (default) or GOM_PRECISION_MIXED */
    int32_t turbulence_flag;   /* i_turbulence_flag of turbulence_closure_v1.f90: 0 off (Av, Kv keep
                                  their values, as in the reference time loop), 1 step function of
                                  the Richardson number, 2 Pacanowski-Philander */
    int32_t transport_solver;  /* C7 transport_solver: 0 or 1 TVD (solve_transport_equation_v19),
                                  2 ELM (solve_transport_equation_ELM_v8) */
    /* Pacanowski-Philander coefficients (h1_pp, h2_pp, vdmax_pp1, vdmax_pp2, vdmin_pp1, vdmin_pp2,
       tdmin_pp of mod_global_variables.f90:909-910) */
    double pp_h1, pp_h2, pp_vdmax1, pp_vdmax2, pp_vdmin1, pp_vdmin2, pp_tdmin;
} gom_params;

/* Arithmetic of a context (no reference counterpart: the reference is FP64 throughout).
 *   GOM_PRECISION_FP64   every state array and every operation in FP64, the reference's order;
 *   GOM_PRECISION_MIXED  layered state (velocities, thicknesses, tracers, momentum coefficients)
 *                        stored and computed in FP32; elevations, the free-surface system and its
 *                        solve, densities, ELM foot coordinates and conservation sums in FP64.
 * The host interface is the same for both: gom_set_field / gom_get_field take and return FP64
 * arrays and convert on the way. */
#define GOM_PRECISION_FP64 0
#define GOM_PRECISION_MIXED 1

/* ------------------------------------------------------------------ static geometry
 * Produced once on the host by read_node_inp/read_cell_inp, set_geometry_1, set_geometry_2,
 * calculate_voronoi_center and calculate_coriolis_factor.  Copied at gom_create. */
typedef struct gom_geom {
    /* nodes */
    const double  *x_node, *y_node, *h_node;             /* (N_n)               */
    const int32_t *adj_cells_at_node;                    /* (N_n)               */
    const int32_t *adj_cellnum_at_node;                  /* (max_nb, N_n)       */
    const int32_t *node_count_each_element;              /* (max_nb, N_n)       */
    const int32_t *adj_nodes_at_node;                    /* (N_n)               */
    const int32_t *adj_nodenum_at_node;                  /* (0:max_nb, N_n)     */
    const int32_t *bottom_layer_at_node;                 /* (N_n)               */
    const int32_t *initial_wetdry_node;                  /* (N_n)               */
    /* cells */
    const double  *x_cell, *y_cell, *h_cell, *area;      /* (N_c)               */
    const int32_t *tri_or_quad;                          /* (N_c)               */
    const int32_t *nodenum_at_cell;                      /* (4, N_c)            */
    const int32_t *facenum_at_cell;                      /* (4, N_c)            */
    const int32_t *adj_cellnum_at_cell;                  /* (4, N_c)            */
    const int32_t *sign_in_outflow;                      /* (4, N_c)            */
    const int32_t *bottom_layer_at_element;              /* (N_c)               */
    const int32_t *ob_element_flag;                      /* (N_c)               */
    const int32_t *qb_element_flag;                      /* (N_c) Qb_element_flag */
    /* faces */
    const double  *x_face, *y_face, *h_face, *face_length, *delta_j;   /* (N_f)   */
    const double  *cos_theta, *sin_theta, *cos_theta2, *sin_theta2;    /* (N_f)   */
    const int32_t *adj_cellnum_at_face;                  /* (2, N_f)            */
    const int32_t *nodenum_at_face;                      /* (2, N_f)            */
    const int32_t *bottom_layer_at_face;                 /* (N_f)               */
    const int32_t *boundary_type_of_face;                /* (N_f) -1 land, 0 inner, >0 open bnd */
    const int32_t *isflowside3;                          /* (N_f) river face -> Q index */
    const double  *coriolis_factor;                      /* (N_f)               */
    const double  *manning;                              /* (N_f) bf_flag 1, may be NULL */
    const double  *bf_height;                            /* (N_f) bf_flag 2, may be NULL */
    /* boundaries */
    const int32_t *ob_cell_id;                           /* (n_ob)              */
    const int32_t *qb_cell;                              /* (n_qb) Q_boundary(:,1) */
    const int32_t *qb_face;                              /* (n_qb) Q_boundary(:,2) */
    /* vertical grid */
    const double  *z_level;                              /* (0:L)               */
    const double  *delta_z;                              /* (L)                 */
    /* packed runs (n_runs > 1, else NULL): 0-based first cell / face / node / open-boundary cell
       of each run, n_runs + 1 entries each, the last being the total */
    const int32_t *run_cell_start, *run_face_start, *run_node_start, *run_ob_start;
} gom_geom;

/* ------------------------------------------------------------------ per-step forcing
 * Computed on the host by setup_spinup, compute_boundary_eta, calculate_Q and the series
 * interpolation at solve_transport_equation_v19.f90:229-534.  NULL array = keep the last
 * uploaded value (all start at zero). */
typedef struct gom_forcing {
    double elapsed_time;               /* it*dt                                      */
    double spinup_tide;                /* spinup_function_tide                       */
    double spinup_baroclinic;          /* spinup_function_baroclinic                 */
    double reserved;
    const double *eta_at_ob_old;       /* (n_ob)                                     */
    const double *eta_at_ob_new;       /* (n_ob)                                     */
    const double *q_add;               /* (n_qb) river discharge Q_add [m3/s]        */
    const double *wind_stress_normal;  /* (N_f) kinematic stress along face normal   */
    const double *wind_stress_tangnt;  /* (N_f)                                      */
    const double *gamma_t;             /* (N_f) surface drag Gamma_T                 */
    const double *air_p;               /* (N_n) air_p1                               */
    const double *con_at_ob;           /* (n_ob, 2, Nt): con_at_ob(i,i3) per subcycle */
    const double *con_at_qb;           /* (n_qb, 2, Nt): con_at_Qb(i,i3) per subcycle */
    const double *phi_sw;              /* (N_c) surface heat term of heat_option 2   */
    const double *phi_sz;              /* (L, N_c) heat source per layer of heat_option 1 and of the
                                          ELM transport (phi_sz of heat_term_by_term.f90), W/m2 */
} gom_forcing;

/* ------------------------------------------------------------------ state fields
 * Shapes are those of mod_global_variables; gom_field_info() returns element count and
 * element size so a caller can size buffers. */
typedef enum gom_field {
    GOM_F_ETA_CELL = 1,        /* (N_c)        */
    GOM_F_ETA_CELL_NEW,        /* (N_c)        */
    GOM_F_ETA_NODE,            /* (N_n)        */
    GOM_F_WETDRY_NODE,         /* (N_n) int    */
    GOM_F_UN_FACE,             /* (L, N_f)     */
    GOM_F_VN_FACE,             /* (L, N_f)     */
    GOM_F_UN_FACE_NEW,         /* (L, N_f)     */
    GOM_F_VN_FACE_NEW,         /* (L, N_f)     */
    GOM_F_UN_ELM,              /* (L, N_f)     */
    GOM_F_VN_ELM,              /* (L, N_f)     */
    GOM_F_WN_CELL,             /* (0:L, N_c)   */
    GOM_F_WN_CELL_NEW,         /* (0:L, N_c)   */
    GOM_F_U_NODE,              /* (0:L, N_n)   */
    GOM_F_V_NODE,              /* (0:L, N_n)   */
    GOM_F_W_NODE,              /* (0:L, N_n)   */
    GOM_F_U_FACE_LEVEL,        /* (0:L, N_f)   */
    GOM_F_V_FACE_LEVEL,        /* (0:L, N_f)   */
    GOM_F_DZ_CELL,             /* (L, N_c)     */
    GOM_F_DZ_CELL_NEW,         /* (L, N_c)     */
    GOM_F_DZHALF_CELL,         /* (0:L, N_c)   */
    GOM_F_DZHALF_CELL_NEW,     /* (0:L, N_c)   */
    GOM_F_DZ_FACE,             /* (L, N_f)     */
    GOM_F_DZ_FACE_NEW,         /* (L, N_f)     */
    GOM_F_DZHALF_FACE,         /* (0:L, N_f)   */
    GOM_F_DZHALF_FACE_NEW,     /* (0:L, N_f)   */
    GOM_F_DZ_NODE,             /* (L, N_n)     */
    GOM_F_DZ_NODE_NEW,         /* (L, N_n)     */
    GOM_F_DZHALF_NODE,         /* (0:L, N_n)   */
    GOM_F_DZHALF_NODE_NEW,     /* (0:L, N_n)   */
    GOM_F_TOP_LAYER_CELL,      /* (N_c) int    */
    GOM_F_TOP_LAYER_FACE,      /* (N_f) int    */
    GOM_F_TOP_LAYER_NODE,      /* (N_n) int    */
    GOM_F_AINVG1,              /* (L, N_f) top-down rows */
    GOM_F_AINVG2,              /* (L, N_f)     */
    GOM_F_AINVDZ1,             /* (L, N_f)     */
    GOM_F_AINVDZ2,             /* (L, N_f)     */
    GOM_F_KH,                  /* (L, N_f)     */
    GOM_F_AV,                  /* (0:L, N_f)   */
    GOM_F_KV,                  /* (0:L, N_c)   */
    GOM_F_SALT_CELL,           /* (L, N_c)     */
    GOM_F_SALT_CELL_NEW,       /* (L, N_c)     */
    GOM_F_TEMP_CELL,           /* (L, N_c)     */
    GOM_F_TEMP_CELL_NEW,       /* (L, N_c)     */
    GOM_F_SALT_NODE,           /* (L, N_n)     */
    GOM_F_TEMP_NODE,           /* (L, N_n)     */
    GOM_F_SALT_FACE,           /* (L, N_f)     */
    GOM_F_TEMP_FACE,           /* (L, N_f)     */
    GOM_F_RHO_CELL,            /* (L, N_c)     */
    GOM_F_RHO_NODE,            /* (L, N_n)     */
    GOM_F_RHO_FACE,            /* (L, N_f)     */
    GOM_F_NUM_SUB_ELM,         /* (L, N_n) int num_sub_elm_iteration */
    GOM_F_CDB,                 /* (N_f)        */
    GOM_F_GAMMA_B,             /* (N_f)        */
    GOM_F_QU_BOUNDARY,         /* (n_qb)       */
    GOM_F_ELM_FOOT,            /* (L, N_f) int: element holding the final ELM foot, 0 = no walk */
    GOM_F_ELM_NEAR_EDGE,       /* (L, N_f) int: 1 if a foot landed within 1e-12 m of an edge    */
    /* per-step forcing arrays (gom_set_forcing uploads them; with storms set the device writes
       them every step) */
    GOM_F_WIND_STRESS_NORMAL,  /* (N_f)        */
    GOM_F_WIND_STRESS_TANGNT,  /* (N_f)        */
    GOM_F_GAMMA_T,             /* (N_f)        */
    GOM_F_AIR_P,               /* (N_n)  Pa    */
    GOM_F_ETA_AT_OB_OLD,       /* (n_ob)       */
    GOM_F_ETA_AT_OB_NEW,       /* (n_ob)       */
    GOM_F_Q_ADD,               /* (n_qb)  m3/s */
    GOM_F_PHI_SW,              /* (N_c)   W/m2 */
    GOM_F_PHI_SZ,              /* (L, N_c) W/m2 */
    GOM_F_COUNT
} gom_field;

/* ------------------------------------------------------------------ entry points */

/* ABI version of the loaded library; must equal GOM_ABI_VERSION. */
int gom_abi_version(void);

/* Human-readable name of an error code (static storage). */
const char *gom_errstr(int code);

/* Last diagnostic message of a context (static to the context; "" if none). */
const char *gom_last_message(const struct gom_ctx *ctx);

/* Element count and element size (8 or 4 bytes) of a field for these dims. */
int gom_field_info(const gom_dims *dims, int field, int64_t *count, int32_t *elem_bytes);

/* Create a context: validates dims/params, copies geometry to the device.
 * Replaces the allocation part of allocate_variables.f90 for the hot-path arrays.
 * The caller then uploads the initial state with gom_set_field (cold or hot start).
 * Limits: n_layers <= 64, n_cells and n_faces below 2^26 (GOM_E_ARG otherwise). */
int gom_create(const gom_dims *dims, const gom_params *params, const gom_geom *geom,
               struct gom_ctx **out);
void gom_destroy(struct gom_ctx *ctx);

/* Upload / download one state field (count elements, checked against the dims). */
int gom_set_field(struct gom_ctx *ctx, int field, const void *host, int64_t count);
int gom_get_field(struct gom_ctx *ctx, int field, void *host, int64_t count);

/* Per-step host forcing (main.f90:85-161). */
int gom_set_forcing(struct gom_ctx *ctx, const gom_forcing *forcing);

/* One entry per reference subroutine of the time loop, in main.f90 order. */
int gom_step_bottom_friction(struct gom_ctx *ctx);   /* calculate_bottom_friction.f90:9      */
int gom_step_boundary_velocity(struct gom_ctx *ctx); /* compute_boundary_velocity.f90:8      */
int gom_step_advection(struct gom_ctx *ctx);         /* solve_nonlinear_advection.f90:14 / main.f90:167-177 */
int gom_step_momentum(struct gom_ctx *ctx);          /* solve_momentum_equation.f90:15      */
int gom_step_free_surface(struct gom_ctx *ctx, int32_t *pcg_iters); /* solve_free_surface_equation.f90:17 */
int gom_step_velocities(struct gom_ctx *ctx);        /* solve_velocities.f90:8               */
int gom_step_layers(struct gom_ctx *ctx);            /* update_vertical_layers_1.f90:18      */
int gom_step_node_velocity(struct gom_ctx *ctx);     /* calculate_velocity_at_node.f90:10    */
int gom_step_transport(struct gom_ctx *ctx);         /* solve_transport_equation_v19.f90:7   */
int gom_step_density(struct gom_ctx *ctx);           /* calculate_density_full.f90:13 / _linear.f90:10 */
int gom_step_turbulence(struct gom_ctx *ctx);        /* turbulence_closure_v1.f90:9 (schemes 1, 2) */
int gom_step_swap(struct gom_ctx *ctx);              /* update_variables.f90:4 (state part)  */

/* The whole per-timestep core after forcing, main.f90:94-272 order, with the turbulence closure
 * (when turbulence_flag != 0) after the density update.  The CUDA library replays it as a
 * captured CUDA graph.  pcg_iters may be NULL. */
int gom_step_all(struct gom_ctx *ctx, int32_t *pcg_iters);

/* gom_step_all split in two, so that many contexts (one per run of an ensemble, each with its own
 * stream) can have a step in flight at once: gom_step_launch enqueues the step and returns;
 * gom_step_wait waits for it and returns its status.  gom_set_forcing may stage the next step's
 * forcing while one step is in flight. */
int gom_step_launch(struct gom_ctx *ctx);
int gom_step_wait(struct gom_ctx *ctx, int32_t *pcg_iters);

/* Device-side storm-surge forcing (no single reference counterpart: it moves onto the GPU what
 * the Fortran driver computes on the host each step in setup_spinup.f90, compute_boundary_eta.f90,
 * holland_storm_surge.f90 and calculate_wind_stress.f90).  One storm per run of the context
 * (n_runs of gom_dims, 1 for a single run).  Once set, every step of the context first advances
 * the elapsed time by dt on the device, then evaluates for each run at that time: a Holland
 * vortex moving on a straight track (the gradient wind of holland_storm_surge.f90:131-188 with a
 * Holland exponent b, 0.95 gradient-to-surface factor, 18 degree inflow, translation asymmetry),
 * air pressure p_far - dp (1 - exp(-(rmax/r)^b)) at the nodes, face wind stress by the drag law
 * of calculate_wind_stress.f90:105-137, and the open-boundary elevation = tide + inverse
 * barometer, all ramped by tanh(2 t / spinup) as setup_spinup.f90 ramps the tide.  gom_set_forcing
 * is then needed only for what the storms leave alone (boundary tracer concentrations). */
typedef struct gom_storm {
    double x0, y0;             /* eye position at elapsed time 0 (m, mesh coordinates) */
    double heading;            /* direction of travel (radians from +x)                */
    double speed;              /* translation speed (m/s)                              */
    double rmax;               /* radius of maximum winds (m)                          */
    double dp;                 /* central pressure deficit (Pa, > 0)                   */
    double b;                  /* Holland exponent                                     */
    double coriolis;           /* Coriolis parameter at the eye (1/s)                  */
    double tide_amplitude;     /* open-boundary tide (m)                               */
    double tide_period;        /* (s)                                                  */
    double tide_phase;         /* (rad)                                                */
    double spinup;             /* ramp period (s); 0 = none                            */
    double t0;                 /* context elapsed time at which this run's clock is 0  */
} gom_storm;
int gom_set_storms(struct gom_ctx *ctx, int32_t n_storms, const gom_storm *storms, double elapsed_time);

/* Boundary series evaluated on the device (no single reference counterpart: it moves onto the
 * GPU what the Fortran driver computes on the host every step in setup_spinup.f90,
 * compute_boundary_eta.f90 (ob_eta_type -1 interior mean, 1 harmonic, 2 time series), calculate_Q.f90 and the
 * boundary-concentration interpolation of solve_transport_equation_v19.f90:229-397).  The tables
 * are the ones read_harmonic_ser.f90, read_eta_ser.f90, read_q_ser.f90, read_salt_ser.f90 and
 * read_temp_ser.f90 hold.  Once set, every gom_step_all / gom_step_launch first advances the
 * device clock (it = it + 1, elapsed_time = it dt, julian_day = julian_day + dt / 86400), forms the
 * spin-up factors, eta_at_ob_old / eta_at_ob_new, Q_add and the boundary salinity and temperature
 * of every transport subcycle, with the reference's expressions (linear interpolation on series
 * times minus reference_diff_days x 86400); a time outside a series keeps the value that entry
 * had.  An open-boundary cell of type -1 with no interior cell around its nodes records GOM_E_ARG
 * in the step status (the reference stops there).  Single-run contexts only.  The separate
 * gom_step_* entry points do not run it.  Station wind, hurricane frames and the heat balance
 * (the fields below) are evaluated the same way, the heat terms just before the transport.
 * gom_set_forcing is then needed only for what the series leave alone (with none of those: wind
 * stress, Gamma_T, air pressure, heat terms).  Not with gom_set_storms on the same context
 * (GOM_E_ARG). */
typedef struct gom_series {
    int32_t n_series;          /* number of series                                          */
    int32_t reserved;
    const int32_t *start;      /* (n_series + 1) offsets of each series in time / value      */
    const double *time;        /* seconds, as the readers store them: (t + adjust) x conv    */
    const double *value;       /* (v + adjust) x conv                                        */
} gom_series;

typedef struct gom_boundary_series {
    double julian_day;              /* julian_day before the next step (prepare_gom.f90:29)    */
    double tide_spinup_period;      /* card C21, days                                           */
    double baroclinic_spinup_period;/* card C21, days                                           */
    int32_t step;                   /* it of the last step taken (the next one is step + 1)     */
    int32_t reference_diff_days;    /* calculate_reference_diff_days.f90                        */
    int32_t tide_spinup;            /* card C21 flag                                            */
    int32_t baroclinic_spinup;      /* card C21 flag (used with baroclinic_flag 1)              */
    int32_t q_interp_method;        /* 1 linear, 2 second-order Lagrange (calculate_Q.f90)      */
    int32_t n_harmonic;             /* harmonic series (num_harmonic_ser)                       */
    const int32_t *ob_eta_type;     /* (n_ob) -1 mean of the interior cells around (old level
                                       only), 1 harmonic, 2 time series, 0 and 3 left as set     */
    const int32_t *ob_harmonic_id;  /* (n_ob) 1-based series ids, 0 none                        */
    const int32_t *ob_eta_id;
    const int32_t *ob_salt_id;
    const int32_t *ob_temp_id;
    const int32_t *qb_q_id;         /* (n_qb) 1-based series ids, 0 none                        */
    const int32_t *qb_salt_id;
    const int32_t *qb_temp_id;
    const double *qb_portion;       /* (n_qb) Q_portion                                         */
    const int32_t *harmonic_start;  /* (n_harmonic + 1) offsets into the constituent arrays      */
    const double *amplitude;        /* per constituent: tidal_amplitude (m)                     */
    const double *period_h;         /* tidal_period (h)                                         */
    const double *nodal;            /* tidal_nodal_factor                                       */
    const double *eq_arg;           /* equilibrium_argument (degrees)                           */
    const double *phase;            /* tidal_phase (degrees)                                    */
    const double *phase_shift;      /* (n_harmonic) tidal_phase_shift (degrees)                 */
    gom_series eta, q, salt, temp;
    /* station wind (card C30, windp_ser.inp): get_windp_at_face.f90 (one station uniform, two or
     * three by inverse distance to their nodes, IDW_windp_ser.f90) and calculate_wind_stress.f90
     * (heat_model_flag 0) form wind_stress_normal / tangnt and Gamma_T every step; with wind_flag
     * 0 the wind arrays are left as gom_set_forcing set them */
    int32_t wind_flag;              /* 1: station wind series                                   */
    int32_t wind_formular;          /* 1, 2 or 3 (the drag-coefficient formula)                 */
    int32_t wind_spinup;            /* flag                                                     */
    int32_t n_wind;                 /* num_windp_ser: 1..3 stations                             */
    double wind_spinup_period;      /* days                                                     */
    double rho_a;                   /* card C1 air density (kg/m3)                              */
    const int32_t *wind_station_node; /* (n_wind) windp_station_node                            */
    gom_series wind_u, wind_v;      /* per station: windp_u, windp_v on windp_ser_time          */
    /* hurricane wind fields (card C31: hurricane_flag 1): node frames of hurricane_ser.inp taken
     * every hurricane_read_interval steps while julian_day lies in [hurricane_start_jday,
     * hurricane_end_jday] (main.f90:115-127).  Between two reads the node winds and air pressure
     * step linearly (hurricane_interp_method 1, read_hurricane_ser_1.f90) or are the two frames
     * moved with the storm centre and blended (method 2, read_hurricane_ser_2.f90 with IDW_5.f90
     * over the neighbour lists of find_neighbour_nodes.f90, built on the device); face winds are
     * their node means, and every step forms the hurricane drag law of
     * calculate_wind_stress.f90:105-137 (Cda <= 0.003) into wind_stress_normal / tangnt and
     * Gamma_T, and air_p from the node pressure.  Each frame after the first two comes from
     * gom_push_hurricane_frame, each centre after the first two (method 2) from
     * gom_push_hurricane_center. */
    int32_t hurricane_flag;         /* 1: hurricane node frames                                 */
    int32_t hurricane_read_interval;/* int(hurricane_dt / dt) >= 1 (read_hurricane_ser_0.f90:27) */
    double hurricane_start_jday;    /* find_hurricane_start_end_jday                            */
    double hurricane_end_jday;
    const double *hurricane_frames; /* (N_n, 3, 3): (wind_u, wind_v, air_p in Pa) of frames 0, 1
                                       and 2 = wind_u0.., wind_u1.., wind_u2.. as the driver holds
                                       them (after read_hurricane_ser_0 frame 1 is all zero)    */
    int32_t hurricane_interp_method;/* 1 (or 0) linear in time, 2 moved with the storm centre     */
    int32_t reserved_hurricane;
    double hurricane_track[6];      /* method 2: hurric_x_1, hurric_y_1, hurricane_time_1,
                                       hurric_x_2, hurric_y_2, hurricane_time_2 (julian days)   */
    /* heat balance (heat_option 1 with temperature transport, heat_term_by_term.f90): every step,
     * before the transport, the air series of air_ser.inp interpolated at julian_day, the
     * short-wave term (sol_swr 1: from the sun's elevation at the local hour of
     * julian_to_localtime.f90; sol_swr 2: from the series), the long-wave, back-radiation,
     * evaporation and conduction terms, and phi_sz (per wet layer) and phi_sw from the top and
     * bottom temperatures and the layer thicknesses; with heat_flag 0 phi_sz / phi_sw are left as
     * gom_set_forcing set them */
    int32_t heat_flag;              /* 1: form phi_sz and phi_sw on the device                  */
    int32_t sol_swr;                /* 1: from the solar elevation, 2: from the air series      */
    int32_t n_air;                  /* samples of air_ser.inp                                   */
    int32_t reserved_heat;
    double fwz_a, fwz_b, fwz_c, wind_height;                               /* card C7_3 */
    double light_extinction, sol_absorb, sed_water_exchange, t_sed, sed_temp_coeff;   /* C7_4 */
    const double *air_time;         /* (n_air) air_ser_time (s, as read_air_ser.f90 stores it)  */
    const double *air_values;       /* (n_air, 5): T_air, T_dew, air_wind_speed,
                                       solar_radiation, cloud                                   */
    int32_t year;                   /* sol_swr 1: the driver's year (card C3 start year) and     */
    int32_t month;                  /* its month variable before the next step                   */
    double lon, lat;                /* card C1 (degrees)                                         */
} gom_boundary_series;
int gom_set_boundary_series(struct gom_ctx *ctx, const gom_boundary_series *series);

/* The next hurricane_ser.inp record, (N_n, 3): wind_u, wind_v, air_p in Pa (the x 100 of
 * read_hurricane_ser_1.f90:37-45 applied).  The device takes it at the next step whose
 * it mod hurricane_read_interval is 0 inside the window; call once before each such step.  A read
 * step with no record pushed records GOM_E_ARG in the step status and keeps the frame it has.
 * Ordered on the context's stream: a record may be pushed while earlier steps still run.
 * Replaces the record read of read_hurricane_ser_1.f90:34-46. */
int gom_push_hurricane_frame(struct gom_ctx *ctx, const double *frame);

/* Method 2: the next hurricane_center record (its x, y and julian day, as julian.f90 converts
 * it), taken with the next frame at the next read step (read_hurricane_ser_2.f90:38-45); call
 * once before each read step.  A read step with no centre pushed records GOM_E_ARG in the step
 * status.  GOM_E_ARG unless the context holds method-2 hurricane frames. */
int gom_push_hurricane_center(struct gom_ctx *ctx, double x, double y, double julian_day);

/* ------------------------------------------------------------------ mesh geometry on the device
 * The start-up geometry of GOM built on the GPU: the areas of read_cell_inp.f90:54-87,
 * set_geometry_1.f90 (node-cell and node-node adjacency, cell-cell adjacency, face numbering,
 * face and cell centres, sign_in_outflow, delta_j, face angles), calculate_voronoi_center.f90
 * (voronoi 1) and set_geometry_2.f90 (open-boundary cells and faces, boundary_type_of_face, bottom
 * layers) plus the river cells and faces of read_main_inp.f90:810-829 and initial_wetdry_node of
 * read_node_inp.f90:72-74.  Integer arrays and every double computed with + - x / and sqrt equal
 * the reference's loops bit for bit; the four angle arrays come from CUDA's atan2 / cos / sin,
 * which may differ from the C library's in the last bit or two. */
typedef struct gom_mesh {
    int32_t n_nodes, n_cells, max_nb, voronoi;
    int32_t n_layers, n_ob, n_qb, reserved;
    const double *x_node, *y_node, *h_node;   /* (N_n) node.inp                                  */
    const int32_t *tri_or_quad;               /* (N_c) cell.inp                                  */
    const int32_t *nodenum_at_cell;           /* (4, N_c) CCW nodes, 1-based, 0 in slot 4 of triangles */
    const double *z_level;                    /* (0:L) card C2 / C2_1                            */
    double msl;
    const int32_t *ob_nodes;                  /* (2, n_ob) node pairs of card C20_1 (CCW)         */
    const int32_t *qb_nodes;                  /* (2, n_qb) node pairs of card C22_1 (CCW)         */
} gom_mesh;

/* Outputs, in host memory the caller owns, laid out as gom_geom takes them.  Face arrays hold
 * face_capacity entries (sum of tri_or_quad bounds the face count); n_faces receives maxface.
 * A NULL array is not written. */
typedef struct gom_mesh_geometry {
    int32_t face_capacity;
    int32_t n_faces;                          /* out                                             */
    int32_t *adj_cells_at_node, *adj_cellnum_at_node, *node_count_each_element;
    int32_t *adj_nodes_at_node, *adj_nodenum_at_node, *bottom_layer_at_node, *initial_wetdry_node;
    double *x_cell, *y_cell, *h_cell, *area;
    int32_t *facenum_at_cell, *adj_cellnum_at_cell, *sign_in_outflow, *bottom_layer_at_element;
    int32_t *ob_element_flag, *qb_element_flag;
    double *x_face, *y_face, *h_face, *face_length, *delta_j;
    double *cos_theta, *sin_theta, *cos_theta2, *sin_theta2;
    int32_t *adj_cellnum_at_face, *nodenum_at_face, *bottom_layer_at_face, *boundary_type_of_face, *isflowside3;
    int32_t *ob_cell_id, *ob_face_id, *qb_cell, *qb_face;   /* (n_ob), (n_qb)                 */
} gom_mesh_geometry;

/* Sites recorded in gom_status.site when gom_geometry_build rejects a mesh (GOM_E_ARG), one per
 * reference `stop`; entity is the smallest offending 1-based index of the first failing check. */
enum {
    GOM_GEO_CONCAVE = 1,          /* read_cell_inp.f90:76-79 (cell)                   */
    GOM_GEO_AREA = 2,             /* read_cell_inp.f90:83-86 (cell)                   */
    GOM_GEO_MAX_NB = 3,           /* set_geometry_1.f90:119-123 (node)                */
    GOM_GEO_HANGING = 4,          /* set_geometry_1.f90:130-134 (node)                */
    GOM_GEO_SURROUNDING = 5,      /* set_geometry_1.f90:178-182 (node)                */
    GOM_GEO_FACE_COUNT = 6,       /* set_geometry_1.f90:254-257                       */
    GOM_GEO_FACE_LENGTH = 7,      /* set_geometry_1.f90:321-324 (face)                */
    GOM_GEO_BALL = 8,             /* set_geometry_1.f90:338-341 (cell)                */
    GOM_GEO_VORONOI = 9,          /* calculate_voronoi_center.f90:58-64 (cell)        */
    GOM_GEO_CENTRES = 10,         /* set_geometry_1.f90:466-469, calculate_voronoi_center.f90:121-124 (face) */
    GOM_GEO_BOUNDARY = 11,        /* set_geometry_2.f90:37-41, read_main_inp.f90:810-822 (ob i, river n_ob + i) */
    GOM_GEO_VERTICAL = 12         /* set_geometry_2.f90:101-189 (entity_kind: cell, face or node) */
};

/* Build the geometry of `mesh` on the current device (its own temporary device memory, freed
 * before return) and copy it into `out`.  GOM_E_ARG for a bad argument or a mesh the reference
 * stops on (failure, if not NULL, receives the site and entity). */
int gom_geometry_build(const gom_mesh *mesh, gom_mesh_geometry *out, gom_status *failure);

/* Cold start computed on the device (no reference counterpart as one routine: it is what
 * setup_cold_start.f90 + update_vertical_layers_0.f90 + uniform read_salt_init.f90 /
 * read_temp_init.f90 leave before the time loop): zero elevation and motion, first layers and
 * thicknesses from the bathymetry, uniform salinity and temperature at cells, faces and nodes,
 * Av = av_0 and Kv = kv_0 at levels 1..L, ELM substeps as card C5_01 sets them.  Densities are
 * left at zero: call gom_step_density next, as prepare_gom does.  For contexts too large to
 * upload a host-built initial state field by field. */
int gom_cold_start(struct gom_ctx *ctx, double salt, double temp, double av_0, double kv_0);

/* Autotuner (no reference counterpart): times the compiled variants of the tunable launches
 * (ELM walk: one thread per face or per listed wet face-layer, threads per block, register
 * budget; momentum columns, transport column solve and limiter: threads per block) on the
 * context's current state, `reps` runs each, keeps the
 * fastest and re-captures the step graph.  The phases it runs only overwrite arrays that the
 * next step recomputes before reading them (ELM velocities, momentum coefficients, transport
 * outputs), so the run's results do not change.  Call between steps.  choice (may be NULL)
 * receives the variant picked per site. */
#define GOM_TUNE_SITES 4
int gom_autotune(struct gom_ctx *ctx, int32_t reps, int32_t *choice);

/* Number of compiled variants per tunable site (no reference counterpart). */
int gom_tuning_variants(int32_t counts[GOM_TUNE_SITES]);

/* Select the variant of each tunable site, e.g. an earlier gom_autotune result reused for a mesh
 * of the same shape (no reference counterpart); -1 keeps a site's current variant, GOM_E_ARG for
 * a variant out of range.  Every variant computes the same results bit for bit. */
int gom_set_tuning(struct gom_ctx *ctx, const int32_t choice[GOM_TUNE_SITES]);

/* Copy every state array of one run of src into one run of dst (no reference counterpart): for
 * moving in-flight runs between packed contexts when a server repacks its ensemble.  The two runs
 * must have the same cell, face and node counts, the contexts the same layers and precision and
 * the same device.  Forcing arrays are not copied (storms recompute them every step). */
int gom_copy_run(struct gom_ctx *dst, int32_t dst_run, struct gom_ctx *src, int32_t src_run);

/* Timing hook for the roofline figures (no reference counterpart): launches one kernel of the
 * step alone `reps` times on the current state and returns its mean time per launch (CUDA
 * events on the context stream).  Call between steps; what it overwrites is recomputed by the
 * next step before it is read. */
#define GOM_KERNEL_ELM_WALK 1         /* the per-face ELM walk                              */
#define GOM_KERNEL_MOMENTUM 2         /* the per-face momentum columns                      */
#define GOM_KERNEL_TRANSPORT_SOLVE 3  /* one TVD transport subcycle's column solve, its    */
                                      /* coefficients formed first (GOM_E_ARG when the     */
                                      /* context has no TVD transport)                     */
int gom_profile_kernel(struct gom_ctx *ctx, int32_t which, int32_t reps, double *ms_per_launch);

/* Device memory the context holds (bytes), for admission by memory budget when many contexts
 * share a GPU. */
int64_t gom_device_bytes(const struct gom_ctx *ctx);

/* Asynchronous output snapshots for the output writers (write_dump3D.f90:4, write_restart.f90:7,
 * write_tser_out_files.f90 read the state between steps; the overlap has no reference
 * counterpart).  gom_snapshot_begin enqueues, after the work already enqueued on the context
 * (a step launched by gom_step_launch included), a copy of the listed fields into a device
 * staging area and their transfer into host[q] (FP64 for real fields whatever the context's
 * precision, int32 for integer fields; sizes as gom_get_field) on a separate copy stream, and
 * returns: the following steps run while the transfer proceeds.  The host buffers should be
 * pinned (gom_host_alloc) for the transfer to overlap, and must not be read before
 * gom_snapshot_wait (blocks until the data has landed) or gom_snapshot_ready (1 landed, 0 still
 * in flight) says so.  One snapshot may be in flight per context (GOM_E_ARG otherwise). */
int gom_snapshot_begin(struct gom_ctx *ctx, int32_t n_fields, const int32_t *fields, void *const *host);
int gom_snapshot_ready(struct gom_ctx *ctx);
int gom_snapshot_wait(struct gom_ctx *ctx);
/* Pinned (page-locked) host memory for snapshot buffers. */
int gom_host_alloc(int64_t bytes, void **out);
void gom_host_free(void *p);

/* Volume and salt mass of the wet cells: sum(area*dz_cell), sum(area*dz_cell*salt_cell),
 * accumulated in FP64 (spec: check_conservation.f90:28-57). */
int gom_conservation(struct gom_ctx *ctx, double *volume, double *salt_mass);

/* Station time series (replaces the state reads of write_tser_out_files.f90:9-330; station ids as
 * read at read_main_inp.f90:1143-1154).  gom_set_stations keeps the station ids on the device:
 * hloc 1 = stations at cells (station_cell used), 2 = at nodes (station_node used), 1-based ids.
 * gom_station_series then gathers, after the work already enqueued, the values the reference
 * writes for every station and waits for them: out is (7 + 4 L, n_stations) FP64, one record per
 * station [eta, H, ubar, u(1:L), vbar, v(1:L), sbar, salt(1:L), tbar, temp(1:L), air pressure],
 * formed as write_tser_out_files.f90 forms them (hloc 1: cell velocities from the node columns,
 * depth means over the wet layers; hloc 2: node columns and the depth means of
 * update_variables.f90:36-72).  Air pressure: hloc 1 reads the per-node air_p at the station's
 * CELL id, as the reference indexes air_p1 (0 where that id exceeds n_nodes); hloc 2 reads air_p at
 * the node (the reference writes airp_at_node there, the wind-series pressure of
 * IDW_windp_ser.f90:97 that the host driver holds).  Call it after gom_step_swap / gom_step_all,
 * where the reference calls write_output_files (main.f90:276). */
int gom_set_stations(struct gom_ctx *ctx, int32_t hloc, int32_t n_stations, const int32_t *station_cell,
                     const int32_t *station_node);
int gom_station_series(struct gom_ctx *ctx, double *out);

/* First recorded failure; clear != 0 resets it. */
int gom_get_status(struct gom_ctx *ctx, gom_status *status, int clear);

/* Wait for all device work of the context. */
int gom_synchronize(struct gom_ctx *ctx);

/* Free-surface Jacobi-PCG solve that allocates nothing (no counterpart in the reference).
 * For callers that cannot call cudaMalloc -- their arrays live in device memory owned by another
 * runtime (OpenACC / CUDA Fortran data regions, a pooled service) -- so they cannot give the
 * solver work vectors.  The work vectors live in a fixed file-scope device array of the library:
 * n_cells must be <= 262144 (GOM_E_ARG otherwise).  Inputs and outputs are device pointers:
 * tri_or_quad (n_cells), adj_cellnum_at_cell (4, n_cells), sparsem (0:4, n_cells: diagonal then
 * the neighbour coefficients in local-face order, as solve_free_surface_equation.f90 builds them),
 * rhs (n_cells), x (n_cells, initial guess in, solution out).  A row whose diagonal is not
 * positive stops the solve with GOM_E_NOT_SPD.  Work is ordered on `stream` (a cudaStream_t,
 * NULL = legacy default stream).  With iterations != NULL the call waits and returns the solve's
 * status and iteration count; with NULL it returns after the launch.  device_result (may be NULL)
 * is device memory for 2 int32 that receive, ordered on `stream`, the solve's status code and
 * iteration count: the way an asynchronous caller learns of a failure (GOM_E_TIMEOUT, GOM_E_NOT_SPD)
 * once it has synchronised `stream`.  All calls share the array: calls that overlap on the GPU race.
 * The solve is a cooperative kernel that spins on grid barriers, so it must not overlap on the GPU
 * with a context's free-surface phase either (order both on one stream, e.g. gom_stream(ctx)).  The
 * first call on a device does a one-time set-up and should come before any stream capture. */
int gom_pcg_solve_noalloc(int32_t n_cells, const int32_t *tri_or_quad, const int32_t *adj_cellnum_at_cell,
                          const double *sparsem, const double *rhs, double *x, int32_t max_iteration,
                          double error_tolerance, void *stream, int32_t *iterations, int32_t *device_result);

/* FP64 arithmetic peak of the current GPU in GFLOP/s (no reference counterpart: the roofline of
 * the plain FP64 path, whose kernels are bound by FP64 issue).  Times one kernel of independent
 * FMA chains with CUDA events; allocates 8 bytes of device memory for the duration of the call.
 * GOM_E_ARG from a CPU implementation. */
int gom_measure_fp64_peak(double *gflops);

/* FP64 warp instructions per second of the current GPU with only the first active_lanes (1..32)
 * lanes of every warp working (no reference counterpart): the same FMA chains as
 * gom_measure_fp64_peak.  On GB300 the rate does not depend on active_lanes, so a warp
 * instruction costs the FP64 pipe the same however many lanes take it.  GOM_E_ARG from a CPU
 * implementation or for a lane count outside 1..32. */
int gom_measure_fp64_issue(int32_t active_lanes, double *warp_instr_per_s);

/* Self-test of the integer comparisons on bit patterns that the kernels use in place of FP
 * comparisons (no reference counterpart): every helper against the FP comparison it stands for,
 * on the device, over all pairs of a table of special and ordinary double and float values
 * (signed zeros, subnormals, infinities, NaNs of both signs).  *checked: comparisons made;
 * *mismatches: those that differed (0 expected).  GOM_E_ARG from a CPU implementation. */
int gom_selftest_compares(int64_t *checked, int64_t *mismatches);

/* The CUDA stream (cudaStream_t) all device work of the context is ordered on, so a caller can
 * record events or order its own work against the core.  NULL for a CPU implementation. */
void *gom_stream(struct gom_ctx *ctx);

/* Accumulated PCG iterations since creation (diagnostic). */
int64_t gom_pcg_iterations_total(struct gom_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif /* GOM_CORE_H */
