/*
 * source_term_host.cu -- the exported source-term functions of the hydroFV
 * API (src/source_term.h:21-31) on the caller's host arrays.
 *
 * launch_simulation never calls them: the step kernels apply the same
 * per-cell updates on the device (the gravity kick in the GRAV build of the
 * 2D step kernel, the geometry source in the 1D run kernel).  Both sides are
 * compiled from the templates in numerics.cuh (geometry_source_rk4,
 * gravity_kick), so a program that calls these functions between its own
 * steps, as the reference's integrators do, gets the GPU path's arithmetic.
 * After the update each function converts U to W over the whole grid and
 * fills the ghost cells, as the reference does.  Host code is compiled with
 * -ffp-contract=off.
 */
#include "hydro.h"
#include "source_term.h"
#include "numerics.cuh"

extern "C" {

/* src/source_term.c:45-183: RK4 of the cylindrical (alpha = 1) or spherical
 * (alpha = 2) geometry source over the interior cells. */
ErrorStatus add_geometry_source_term(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    const double dt
)
{
    double alpha;
    switch (system->coord_sys_flag_) {
    case COORD_SYS_CARTESIAN_1D:
    case COORD_SYS_CARTESIAN_2D:
    case COORD_SYS_CARTESIAN_3D:
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Wrong coordinate system, expected cylindrical 1D or spherical 1D.");
    case COORD_SYS_CYLINDRICAL_1D:
        alpha = 1.0;
        break;
    case COORD_SYS_SPHERICAL_1D:
        alpha = 2.0;
        break;
    default:
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Unknown coordinate system flag.");
    }

    const int g = system->num_ghost_cells_side;
    const int n = system->num_cells_x;
    const double gm1 = system->gamma - 1.0;
    for (int i = g; i < n + g; i++) {
        const double vol = system->volume_[i];
        double m = system->mass_[i], mom = system->momentum_x_[i], E = system->energy_[i];
        hydro::geometry_source_rk4(-alpha * vol / system->mid_points_x_[i], gm1, vol, dt,
                                   system->density_[i], m, mom, E);
        system->mass_[i] = m;
        system->momentum_x_[i] = mom;
        system->energy_[i] = E;
    }

    ErrorStatus e = WRAP_TRACEBACK(convert_conserved_to_primitive(system));
    if (e.return_code != SUCCESS) return e;
    return WRAP_TRACEBACK(set_boundary_condition(boundary_condition_param, system));
}

/* src/source_term.c:185-259: the gravity kick on the interior cells of a 2D
 * grid; nothing happens (not even the conversion) when gravity is zero. */
ErrorStatus add_gravity_source_term_2d(
    const BoundaryConditionParam *__restrict boundary_condition_param,
    System *__restrict system,
    const double dt
)
{
    const double gravity = system->gravity;
    if (gravity == 0.0) return make_success_error_status();

    const int g = system->num_ghost_cells_side;
    const int nx = system->num_cells_x;
    const int ny = system->num_cells_y;
    const int tx = nx + 2 * g;
    const double pf = -dt * gravity;
    for (int j = g; j < ny + g; j++) {
        for (int i = g; i < nx + g; i++) {
            const int idx = j * tx + i;
            hydro::gravity_kick(pf, system->mass_[idx], system->momentum_y_[idx], system->energy_[idx]);
        }
    }

    ErrorStatus e = WRAP_TRACEBACK(convert_conserved_to_primitive(system));
    if (e.return_code != SUCCESS) return e;
    return WRAP_TRACEBACK(set_boundary_condition(boundary_condition_param, system));
}

}  // extern "C"
