/*
 * clshim.h -- inspection calls of the OpenCL shim over the CPU oracle
 * (clshim.c).  TEST INFRASTRUCTURE ONLY.
 */
#ifndef SIMRADAR_CLSHIM_H
#define SIMRADAR_CLSHIM_H

#include <stddef.h>

#include "CL/cl.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The host storage of a buffer or image rs.c created: its bytes and, for an
 * image, its texels per axis (a buffer gives bytes / 16, 1, 1). */
const void *clshim_mem_data(cl_mem m, size_t *bytes, size_t dims[3]);
/* How many launches of the rs.cl kernel `name` the device has run. */
unsigned long long clshim_launches(const char *name);
const char *clshim_last_error(void);

/* The value (or, for a memory argument, the cl_mem) kernel argument `index`
 * holds now; 0 on success. */
int clshim_kernel_arg(cl_kernel k, unsigned index, void *out, size_t size);

/* An observer of what rs.c sends to the device, called before a transfer
 * lands or a kernel runs. */
enum { CLSHIM_WRITE_BUFFER = 1, CLSHIM_WRITE_IMAGE = 2, CLSHIM_LAUNCH = 3 };
typedef struct {
    int kind;
    cl_mem mem;            /* the buffer or image written (transfers) */
    size_t offset, size;   /* bytes (buffer writes) */
    const void *ptr;       /* host data being written */
    cl_kernel kernel;      /* launches */
    const char *name;      /* the kernel's rs.cl name */
    size_t global_offset, global_size, local_size;
} clshim_event;
void clshim_set_hook(void (*hook)(const clshim_event *ev, void *user), void *user);

/* The kernels the device runs: the oracle's restatement (the default) or the
 * reference's own rs.cl compiled for the CPU (rscl.h). */
enum { CLSHIM_KERNELS_ORACLE = 0, CLSHIM_KERNELS_RSCL = 1 };
void clshim_set_kernels(int which);

#ifdef __cplusplus
}
#endif

#endif
