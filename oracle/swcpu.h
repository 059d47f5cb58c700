/*
 * swcpu.h -- CPU oracle for the ANUGA explicit shallow-water Euler step.
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU
 * baseline of bench.py; never linked into the product library.
 *
 * The parameter block and domain block are mirrored field for field by
 * oracle/oracle.py (ctypes); keep the two in step.
 */
#ifndef SWCPU_H
#define SWCPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SWCPU_BC_REFLECTIVE = 0,
    SWCPU_BC_DIRICHLET = 1,
    SWCPU_BC_TIME_STAGE_SINE = 2,
    SWCPU_BC_TRANSMISSIVE = 3,
    SWCPU_BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM = 4,
    SWCPU_BC_INFLOW_HYDROGRAPH = 5,
    SWCPU_BC_TIME_STAGE_FOURIER = 6,
};

enum {
    SWCPU_ERR_DISCONTINUOUS_BED = 1,
    SWCPU_ERR_DENOMINATOR = 2,
    SWCPU_ERR_NO_INTERIOR_NEIGHBOUR = 4,
    SWCPU_ERR_BOUNDARY_TYPE = 8,
    SWCPU_ERR_SMALL_TIMESTEP = 16,
};

/* ANUGA numerical parameters (Domain attributes read by the reference's
 * struct domain, src/anuga_HMPP/sw_domain_fun.h:57-120). */
typedef struct {
    double g;
    double epsilon;
    double H0;
    double minimum_allowed_height;
    double maximum_allowed_speed;
    double beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry;
    double alpha_balance;
    double CFL;
    double evolve_max_timestep;
    double evolve_min_timestep;
    long tight_slope_limiters;
    long use_centroid_velocities;
    long optimise_dry_cells;
    long extrapolate_velocity_second_order;
    long use_sloped_mannings;
    long max_smallsteps;
    long default_order;
    long optimised_gradient_limiter; /* 1: extrapolate_second_order_sw */
    long use_edge_limiter;           /* 1: per-quantity limit by edge */
    long flow_algorithm;             /* 0 default, 1 'tsunami' (protect_swb2 +
                                        edge extrapolation, no balance) */
} swcpu_params;

typedef struct {
    long type;     /* SWCPU_BC_* */
    double p[8];   /* Dirichlet: stage, xmom, ymom; sine: mean, amp, period, phase;
                      hydrograph: peak unit discharge, rise, fall, start time;
                      Fourier: c0..c4, period */
} swcpu_boundary_tag;

typedef struct {
    const swcpu_params *params;
    long number_of_elements;
    long number_of_boundary_elements;

    /* mesh (ANUGA layout, int64 indices) */
    const long *neighbours, *neighbour_edges, *surrogate_neighbours;
    const long *number_of_boundaries, *tri_full_flag;
    const double *normals, *edgelengths, *radii, *areas;
    const double *vertex_coordinates, *centroid_coordinates;
    const long *boundary_cells, *boundary_edges, *boundary_tag;
    const swcpu_boundary_tag *tags;

    /* quantities */
    double *stage_centroid_values, *xmom_centroid_values, *ymom_centroid_values;
    double *bed_centroid_values, *friction_centroid_values;
    double *stage_vertex_values, *xmom_vertex_values, *ymom_vertex_values;
    double *bed_vertex_values;
    double *stage_edge_values, *xmom_edge_values, *ymom_edge_values;
    double *bed_edge_values;
    double *stage_boundary_values, *xmom_boundary_values, *ymom_boundary_values;
    double *bed_boundary_values;
    double *stage_explicit_update, *xmom_explicit_update, *ymom_explicit_update;
    double *stage_semi_implicit_update, *xmom_semi_implicit_update,
        *ymom_semi_implicit_update;
    double *max_speed;

    /* scratch: 3N flags, two N-double stores */
    unsigned char *work_flags;
    double *work_a, *work_b;

    /* evolve state */
    double time, starttime, yieldtime, timestep, flux_timestep;
    double recorded_max_timestep, recorded_min_timestep;
    long order, smallsteps, number_of_steps;
    long status;

    /* Runge-Kutta stepping: 1 euler, 2 rk2, 3 rk3, and the centroid
     * backups of the conserved quantities (N doubles each; only read and
     * written when timestepping_method > 1 or by the backup call) */
    long timestepping_method;
    double *stage_centroid_backup, *xmom_centroid_backup, *ymom_centroid_backup;

    /* edge midpoints [6N] (x, y per edge), for the edge extrapolation */
    const double *edge_coordinates;
} swcpu_domain;

double swcpu_compute_fluxes(swcpu_domain *D);
int swcpu_edge_speeds(const swcpu_domain *D, double *ms_out);
void swcpu_gravity_wb(swcpu_domain *D);
void swcpu_manning_friction(swcpu_domain *D);
int swcpu_update_conserved_quantities(swcpu_domain *D, double dt);
void swcpu_protect(swcpu_domain *D);
void swcpu_extrapolate_second_order_sw(swcpu_domain *D);
void swcpu_extrapolate_first_order(swcpu_domain *D);
int swcpu_extrapolate_and_limit_by_neighbours(swcpu_domain *D, int by_edge);
void swcpu_protect_swb2(swcpu_domain *D);
int swcpu_extrapolate_second_order_edge_sw(swcpu_domain *D);
void swcpu_balance_deep_and_shallow(swcpu_domain *D);
void swcpu_interpolate_to_edges(swcpu_domain *D);
void swcpu_distribute_to_vertices_and_edges(swcpu_domain *D);
void swcpu_update_boundary(swcpu_domain *D);
double swcpu_hydrograph(const double p[4], double t);
void swcpu_update_timestep(swcpu_domain *D, double finaltime);
int swcpu_evolve_one_euler_step(swcpu_domain *D, double finaltime);
void swcpu_backup_conserved_quantities(swcpu_domain *D);
void swcpu_saxpy_conserved_quantities(swcpu_domain *D, double a, double b);
int swcpu_evolve_one_rk2_step(swcpu_domain *D, double finaltime);
int swcpu_evolve_one_rk3_step(swcpu_domain *D, double finaltime);
void swcpu_evolve_start(swcpu_domain *D, double yieldstep);
int swcpu_evolve_steps(swcpu_domain *D, double yieldstep, double finaltime,
                       long max_steps, double time_epsilon);
double swcpu_mass(const swcpu_domain *D);
void swcpu_manning_friction_explicit(swcpu_domain *D);
void swcpu_boundary_velocities_and_height(const swcpu_domain *D, double *h, double *u,
                                          double *v);
/* test knob: pow and sin results moved by n ulps (0: as the host libm) */
void swcpu_set_libm_ulps(int n);
void swcpu_velocities_and_height(const swcpu_domain *D, double *h, double *u,
                                 double *v);

#ifdef __cplusplus
}
#endif
#endif
