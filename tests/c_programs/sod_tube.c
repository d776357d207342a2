/*
 * sod_tube.c -- a C program written against hydro.h the way hydroFV users
 * write them: it sets up the 1000-cell Sod tube, calls launch_simulation
 * and writes the final state.  The GPU tests build it with gcc against
 * include/ and libhydro_gb300.so, run it, and compare its output with the
 * reference's own result for the same problem.
 *
 *   sod_tube <output file> [pressure scale]
 *
 * Output (native byte order): int64 num_steps, double t, double dt, then
 * density, velocity_x, pressure, mass, momentum_x, energy over the padded
 * grid (num_cells_x + 2 * num_ghost_cells_side doubles each).
 *
 * The optional pressure scale multiplies both initial pressures.  At 1e12
 * the exact solver's bisection cannot reach its absolute tolerance and
 * launch_simulation fails; the program then prints the traceback, still
 * writes the state the System holds, and exits with status 3.
 */
#include <stdio.h>
#include <stdlib.h>

#include "hydro.h"

int main(int argc, char **argv)
{
    if (argc != 2 && argc != 3) {
        fprintf(stderr, "usage: %s <output file> [pressure scale]\n", argv[0]);
        return 2;
    }
    const double scale = (argc == 3) ? strtod(argv[2], NULL) : 1.0;

    System system = get_new_system_struct();
    system.coord_sys = "cartesian_1d";
    system.gamma = 1.4;
    system.x_min = 0.0;
    system.x_max = 1.0;
    system.num_cells_x = 1000;
    system.num_ghost_cells_side = 2;
    ErrorStatus status = system_init(&system);
    if (status.return_code != SUCCESS) {
        print_and_free_traceback(&status);
        return 1;
    }

    /* left state (1, 0, 1) for x < 0.5, right (0.125, 0, 0.1), ghost cells included */
    const int total = system.num_cells_x + 2 * system.num_ghost_cells_side;
    for (int i = 0; i < total; i++) {
        const int left = system.mid_points_x_[i] < 0.5;
        system.density_[i] = left ? 1.0 : 0.125;
        system.velocity_x_[i] = 0.0;
        system.pressure_[i] = (left ? 1.0 : 0.1) * scale;
    }
    status = convert_primitive_to_conserved(&system);
    if (status.return_code != SUCCESS) {
        print_and_free_traceback(&status);
        return 1;
    }

    BoundaryConditionParam boundary = get_new_boundary_condition_param();
    boundary.boundary_condition_x_min = "transmissive";
    boundary.boundary_condition_x_max = "transmissive";

    IntegratorParam integrator = get_new_integrator_param();
    integrator.integrator = "godunov_first_order_1d";
    integrator.riemann_solver = "riemann_solver_exact";
    integrator.slope_limiter = "minmod";   /* required by the parameter checks, unused by Godunov */
    integrator.cfl = 0.9;

    StoringParam storing = get_new_storing_param();
    storing.is_storing = false;

    Settings settings;
    settings.verbose = 0;
    settings.no_progress_bar = true;

    SimulationParam simulation;
    simulation.tf = 0.2;

    SimulationStatus simulation_status;
    status = launch_simulation(&boundary, &system, &integrator, &storing, &settings, &simulation,
                               &simulation_status);
    const int failed = status.return_code != SUCCESS;
    if (failed) print_and_free_traceback(&status);

    FILE *f = fopen(argv[1], "wb");
    if (!f) {
        perror(argv[1]);
        free_system_memory(&system);
        return 1;
    }
    const long long steps = (long long) simulation_status.num_steps;
    fwrite(&steps, sizeof steps, 1, f);
    fwrite(&simulation_status.t, sizeof(double), 1, f);
    fwrite(&simulation_status.dt, sizeof(double), 1, f);
    const double *fields[6] = { system.density_, system.velocity_x_, system.pressure_,
                                system.mass_, system.momentum_x_, system.energy_ };
    for (int q = 0; q < 6; q++) fwrite(fields[q], sizeof(double), (size_t) total, f);
    fclose(f);
    free_system_memory(&system);
    return failed ? 3 : 0;
}
