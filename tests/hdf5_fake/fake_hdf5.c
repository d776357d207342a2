/*
 * fake_hdf5.c -- the recording stand-in declared in hdf5.h.  TEST
 * INFRASTRUCTURE ONLY: see hdf5.h.
 *
 * Every object gets an id; a dataset remembers its parent group, name,
 * element type and shape.  H5Dwrite renders the data as text (doubles as
 * exact hexadecimal floats, integers in decimal, variable-length strings
 * quoted), and H5Fclose writes the sorted lines to the path given to
 * H5Fcreate.  One file is open at a time, which is how the writers use it.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hdf5.h"

enum { K_FILE = 1, K_GROUP, K_SPACE, K_TYPE, K_DSET };

typedef struct {
    int kind;
    char name[256];      /* groups and datasets: full path */
    hid_t type;          /* datasets: element type; types: the copied base */
    size_t size;         /* types: H5Tset_size value */
    int rank;            /* spaces */
    hsize_t n;           /* spaces: element count */
    hid_t space;         /* datasets */
} Obj;

#define MAX_OBJ 4096
static Obj g_obj[MAX_OBJ];
static hid_t g_next = 1;
static char g_path[4096];
static char *g_lines[MAX_OBJ];
static int g_nlines = 0;

static hid_t new_obj(int kind)
{
    if (g_next >= MAX_OBJ) return H5I_INVALID_HID;
    memset(&g_obj[g_next], 0, sizeof(Obj));
    g_obj[g_next].kind = kind;
    return g_next++;
}

static void add_line(const char *s)
{
    if (g_nlines < MAX_OBJ) g_lines[g_nlines++] = strdup(s);
}

hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl)
{
    (void) flags; (void) fcpl; (void) fapl;
    snprintf(g_path, sizeof g_path, "%s", name);
    g_nlines = 0;
    hid_t id = new_obj(K_FILE);
    if (id != H5I_INVALID_HID) strcpy(g_obj[id].name, "");
    return id;
}

static int cmp(const void *a, const void *b)
{
    return strcmp(*(char *const *) a, *(char *const *) b);
}

herr_t H5Fclose(hid_t file)
{
    (void) file;
    qsort(g_lines, (size_t) g_nlines, sizeof(char *), cmp);
    FILE *f = fopen(g_path, "w");
    if (!f) return -1;
    for (int i = 0; i < g_nlines; i++) {
        fputs(g_lines[i], f);
        fputc('\n', f);
        free(g_lines[i]);
    }
    g_nlines = 0;
    return fclose(f) == 0 ? 0 : -1;
}

static void join(char *out, size_t len, hid_t loc, const char *name)
{
    if (name[0] == '/') snprintf(out, len, "%s", name);
    else snprintf(out, len, "%s/%s", g_obj[loc].name, name);
}

hid_t H5Gcreate2(hid_t loc, const char *name, hid_t lcpl, hid_t gcpl, hid_t gapl)
{
    (void) lcpl; (void) gcpl; (void) gapl;
    hid_t id = new_obj(K_GROUP);
    if (id == H5I_INVALID_HID) return id;
    join(g_obj[id].name, sizeof g_obj[id].name, loc, name);
    char line[512];
    snprintf(line, sizeof line, "%s\tgroup", g_obj[id].name);
    add_line(line);
    return id;
}

herr_t H5Gclose(hid_t group) { (void) group; return 0; }

hid_t H5Screate(H5S_class_t type)
{
    hid_t id = new_obj(K_SPACE);
    if (id != H5I_INVALID_HID) { g_obj[id].rank = (type == H5S_SCALAR) ? 0 : 1; g_obj[id].n = 1; }
    return id;
}

hid_t H5Screate_simple(int rank, const hsize_t dims[], const hsize_t maxdims[])
{
    (void) maxdims;
    hid_t id = new_obj(K_SPACE);
    if (id == H5I_INVALID_HID) return id;
    g_obj[id].rank = rank;
    g_obj[id].n = 1;
    for (int k = 0; k < rank; k++) g_obj[id].n *= dims[k];
    return id;
}

herr_t H5Sclose(hid_t space) { (void) space; return 0; }

hid_t H5Tcopy(hid_t type)
{
    hid_t id = new_obj(K_TYPE);
    if (id != H5I_INVALID_HID) { g_obj[id].type = type; g_obj[id].size = 1; }
    return id;
}

herr_t H5Tset_size(hid_t type, size_t size) { g_obj[type].size = size; return 0; }
herr_t H5Tclose(hid_t type) { (void) type; return 0; }

hid_t H5Dcreate2(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl, hid_t dapl)
{
    (void) lcpl; (void) dcpl; (void) dapl;
    hid_t id = new_obj(K_DSET);
    if (id == H5I_INVALID_HID) return id;
    join(g_obj[id].name, sizeof g_obj[id].name, loc, name);
    g_obj[id].type = type;
    g_obj[id].space = space;
    return id;
}

static const char *type_name(hid_t t)
{
    if (t == H5T_NATIVE_DOUBLE) return "float64";
    if (t == H5T_NATIVE_LLONG) return "int64";
    if (t == H5T_NATIVE_INT) return "int32";
    if (t > 0 && t < MAX_OBJ && g_obj[t].kind == K_TYPE && g_obj[t].type == H5T_C_S1)
        return g_obj[t].size == H5T_VARIABLE ? "vlen_str" : "fixed_str";
    return "unknown";
}

herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer, const void *buf)
{
    (void) mem_space; (void) file_space; (void) xfer;
    const Obj *d = &g_obj[dset];
    const Obj *s = &g_obj[d->space];
    const char *tn = type_name(d->type);
    const hsize_t n = s->n;
    size_t cap = 512 + (size_t) n * 32;
    char *line = malloc(cap);
    if (!line) return -1;
    size_t at = (size_t) snprintf(line, cap, "%s\t%s\t%s\trank=%d n=%llu\t", d->name, tn, type_name(mem_type),
                                  s->rank, (unsigned long long) n);
    for (hsize_t i = 0; i < n && at < cap; i++) {
        if (d->type == H5T_NATIVE_DOUBLE)
            at += (size_t) snprintf(line + at, cap - at, "%s%a", i ? "," : "", ((const double *) buf)[i]);
        else if (d->type == H5T_NATIVE_LLONG)
            at += (size_t) snprintf(line + at, cap - at, "%s%lld", i ? "," : "", ((const long long *) buf)[i]);
        else if (d->type == H5T_NATIVE_INT)
            at += (size_t) snprintf(line + at, cap - at, "%s%d", i ? "," : "", ((const int *) buf)[i]);
        else
            at += (size_t) snprintf(line + at, cap - at, "%s\"%s\"", i ? "," : "",
                                    ((const char *const *) buf)[i] ? ((const char *const *) buf)[i] : "(null)");
    }
    add_line(line);
    free(line);
    return 0;
}

herr_t H5Dclose(hid_t dset) { (void) dset; return 0; }
