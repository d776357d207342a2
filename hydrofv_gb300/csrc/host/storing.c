/*
 * storing.c -- snapshot parameters and writers.
 *
 * Parameter handling follows src/storing.c:27-218 (defaults, interval
 * check, a snapshots_YYYYMMDD_HHMMSS/ default directory, trailing-slash
 * check, mkdir with an "already exists" warning).
 *
 * Writers: when built with HDF5 (-DHYDRO_WITH_HDF5) a snapshot is the
 * reference's snapshot_<k>.h5 layout (src/storing.c:230-765): groups
 * /simulation_status, /fields (padded primitive arrays, flattened 1D) and
 * /parameters.  Without HDF5 the same content goes to snapshot_<k>.bin, a
 * little-endian raw file: magic "HYDROFV\0", int32 dim, nx, ny, g, int64
 * num_steps, float64 t, dt, then the padded fields density, velocity_x,
 * [velocity_y], pressure as float64.
 *
 * The GPU integrators call store_snapshot with a System view whose primitive
 * arrays point at pinned host buffers filled by an asynchronous device-to-host
 * copy of the materialized state.
 */
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <time.h>

#include "hydro.h"

#ifdef HYDRO_WITH_HDF5
#include <hdf5.h>
#endif

StoringParam get_new_storing_param(void)
{
    StoringParam p;
    memset(&p, 0, sizeof p);
    p.is_storing = false;
    p.store_initial = false;
    p.output_dir = NULL;
    p.storing_interval = -1.0;
    p.store_count_ = 0;
    return p;
}

ErrorStatus finalize_storing_param(StoringParam *__restrict p)
{
    if (!p->is_storing)
    {
        return make_success_error_status();
    }
    if (p->storing_interval <= 0.0)
    {
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Storing interval must be positive.");
    }
    char msg[1024];
    if (!p->output_dir)
    {
        const size_t len = strlen("snapshots_YYYYMMDD_HHMMSS/") + 1;
        char *dir = malloc(len);
        if (!dir)
        {
            return WRAP_RAISE_ERROR(MEMORY_ERROR, "Failed to allocate memory for directory path.");
        }
        const time_t raw = time(NULL);
        struct tm tm_buf;
        localtime_r(&raw, &tm_buf);
        strftime(dir, len, "snapshots_%Y%m%d_%H%M%S/", &tm_buf);
        p->output_dir = dir;
    }
    else if (p->output_dir[0] == '\0' || p->output_dir[strlen(p->output_dir) - 1] != '/')
    {
        snprintf(msg, sizeof msg,
                 "Directory path for storing snapshots must end with a trailing slash (\"/\"). Got: \"%s\".",
                 p->output_dir);
        return WRAP_RAISE_ERROR(VALUE_ERROR, msg);
    }
    if (mkdir(p->output_dir, 0777) == -1)
    {
        struct stat st;
        if (stat(p->output_dir, &st) != 0)
        {
            snprintf(msg, sizeof msg, "Failed to access path for storing snapshots: \"%s\".", p->output_dir);
            return WRAP_RAISE_ERROR(OS_ERROR, msg);
        }
        if (S_ISDIR(st.st_mode))
        {
            snprintf(msg, sizeof msg,
                     "Directory for storing snapshots already exists. The files will be overwritten. Directory: \"%s\".",
                     p->output_dir);
            WRAP_RAISE_WARNING(msg);
        }
        else
        {
            snprintf(msg, sizeof msg, "Failed to create directory for storing snapshots: \"%s\".", p->output_dir);
            return WRAP_RAISE_ERROR(OS_ERROR, msg);
        }
    }
    return make_success_error_status();
}

#ifndef HYDRO_WITH_HDF5
static int write_all(FILE *f, const void *data, size_t bytes)
{
    return fwrite(data, 1, bytes, f) == bytes ? 0 : -1;
}
#endif

ErrorStatus store_snapshot(
    const BoundaryConditionParam *__restrict bcp,
    const System *__restrict s,
    const IntegratorParam *__restrict ip,
    const SimulationStatus *__restrict st,
    StoringParam *__restrict p
)
{
    (void) ip;
    const int flag = s->coord_sys_flag_;
    const int is2d = flag == COORD_SYS_CARTESIAN_2D;
    if (!is2d && flag != COORD_SYS_CARTESIAN_1D && flag != COORD_SYS_CYLINDRICAL_1D &&
        flag != COORD_SYS_SPHERICAL_1D)
    {
        return WRAP_RAISE_ERROR(VALUE_ERROR, "Coordinate system flag not recognized.");
    }
    const int g = s->num_ghost_cells_side;
    const long long total = (long long) (s->num_cells_x + 2 * g) * (is2d ? (s->num_cells_y + 2 * g) : 1);
    char path[4096];
#ifdef HYDRO_WITH_HDF5
    snprintf(path, sizeof path, "%ssnapshot_%d.h5", p->output_dir, p->store_count_);
    hid_t file = H5Fcreate(path, H5F_ACC_TRUNC, H5P_DEFAULT, H5P_DEFAULT);
    if (file == H5I_INVALID_HID)
    {
        return WRAP_RAISE_ERROR(OS_ERROR, "Failed to create HDF5 file.");
    }
    hid_t g_status = H5Gcreate(file, "/simulation_status", H5P_DEFAULT, H5P_DEFAULT, H5P_DEFAULT);
    hid_t g_fields = H5Gcreate(file, "/fields", H5P_DEFAULT, H5P_DEFAULT, H5P_DEFAULT);
    hid_t g_params = H5Gcreate(file, "/parameters", H5P_DEFAULT, H5P_DEFAULT, H5P_DEFAULT);
    hsize_t n = (hsize_t) total;
    hid_t scalar = H5Screate(H5S_SCALAR);
    hid_t field = H5Screate_simple(1, &n, NULL);
    hid_t vstr = H5Tcopy(H5T_C_S1);
    H5Tset_size(vstr, H5T_VARIABLE);
#define PUT(grp, name, type, space, ptr)                                                        \
    do {                                                                                        \
        hid_t d_ = H5Dcreate(grp, name, type, space, H5P_DEFAULT, H5P_DEFAULT, H5P_DEFAULT);   \
        H5Dwrite(d_, type, H5S_ALL, H5S_ALL, H5P_DEFAULT, ptr);                                 \
        H5Dclose(d_);                                                                           \
    } while (0)
    PUT(g_status, "num_steps", H5T_NATIVE_LLONG, scalar, &st->num_steps);
    PUT(g_status, "simulation_time", H5T_NATIVE_DOUBLE, scalar, &st->t);
    PUT(g_status, "dt", H5T_NATIVE_DOUBLE, scalar, &st->dt);
    PUT(g_fields, "density", H5T_NATIVE_DOUBLE, field, s->density_);
    PUT(g_fields, "velocity_x", H5T_NATIVE_DOUBLE, field, s->velocity_x_);
    if (is2d) PUT(g_fields, "velocity_y", H5T_NATIVE_DOUBLE, field, s->velocity_y_);
    PUT(g_fields, "pressure", H5T_NATIVE_DOUBLE, field, s->pressure_);
    PUT(g_params, "x_min", H5T_NATIVE_DOUBLE, scalar, &s->x_min);
    PUT(g_params, "x_max", H5T_NATIVE_DOUBLE, scalar, &s->x_max);
    PUT(g_params, "num_cells_x", H5T_NATIVE_INT, scalar, &s->num_cells_x);
    PUT(g_params, "num_ghost_cells_side", H5T_NATIVE_INT, scalar, &s->num_ghost_cells_side);
    PUT(g_params, "dx", H5T_NATIVE_DOUBLE, scalar, &s->dx_);
    PUT(g_params, "gamma", H5T_NATIVE_DOUBLE, scalar, &s->gamma);
    PUT(g_params, "coordinate_system", vstr, scalar, &s->coord_sys);
    PUT(g_params, "boundary_condition_x_min", vstr, scalar, &bcp->boundary_condition_x_min);
    PUT(g_params, "boundary_condition_x_max", vstr, scalar, &bcp->boundary_condition_x_max);
    if (is2d)
    {
        PUT(g_params, "y_min", H5T_NATIVE_DOUBLE, scalar, &s->y_min);
        PUT(g_params, "y_max", H5T_NATIVE_DOUBLE, scalar, &s->y_max);
        PUT(g_params, "num_cells_y", H5T_NATIVE_INT, scalar, &s->num_cells_y);
        PUT(g_params, "dy", H5T_NATIVE_DOUBLE, scalar, &s->dy_);
        PUT(g_params, "boundary_condition_y_min", vstr, scalar, &bcp->boundary_condition_y_min);
        PUT(g_params, "boundary_condition_y_max", vstr, scalar, &bcp->boundary_condition_y_max);
    }
#undef PUT
    H5Tclose(vstr);
    H5Sclose(field);
    H5Sclose(scalar);
    H5Gclose(g_params);
    H5Gclose(g_fields);
    H5Gclose(g_status);
    H5Fclose(file);
#else
    (void) bcp;
    snprintf(path, sizeof path, "%ssnapshot_%d.bin", p->output_dir, p->store_count_);
    FILE *f = fopen(path, "wb");
    if (!f)
    {
        return WRAP_RAISE_ERROR(OS_ERROR, "Failed to create snapshot file.");
    }
    const char magic[8] = { 'H', 'Y', 'D', 'R', 'O', 'F', 'V', '\0' };
    const int32_t hdr[4] = { is2d ? 2 : 1, s->num_cells_x, is2d ? s->num_cells_y : 1, g };
    const int64_t steps = st->num_steps;
    const double times[2] = { st->t, st->dt };
    int rc = write_all(f, magic, sizeof magic) | write_all(f, hdr, sizeof hdr) |
             write_all(f, &steps, sizeof steps) | write_all(f, times, sizeof times);
    const size_t bytes = (size_t) total * sizeof(double);
    rc |= write_all(f, s->density_, bytes) | write_all(f, s->velocity_x_, bytes);
    if (is2d) rc |= write_all(f, s->velocity_y_, bytes);
    rc |= write_all(f, s->pressure_, bytes);
    if (fclose(f) != 0) rc = -1;
    if (rc)
    {
        return WRAP_RAISE_ERROR(OS_ERROR, "Failed to write snapshot file.");
    }
#endif
    p->store_count_++;
    return make_success_error_status();
}
