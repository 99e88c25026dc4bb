/*
 * clshim.c -- the OpenCL host API subset rs.c calls, implemented on the CPU
 * oracle, so that the reference host (rs.c, compiled unmodified from the
 * reference tree) runs its own code path end to end in this build.
 *
 * TEST INFRASTRUCTURE ONLY.  It is linked into oracle/_ref/ (with rs.c and
 * the reference's les / adm / rcs / obj / pos / log modules) by
 * oracle/ref/Makefile, and used by tests/ and tests/golden/ to obtain what
 * the reference host derives (scan box, gate count, population, table
 * descriptors, per-pulse descriptors) and the pulses and state its kernel
 * sequence produces.  Nothing in the simradar_gb300 package loads it.
 *
 * The one "device" it offers runs each rs.cl kernel rs.c enqueues with the
 * oracle's restatement of that kernel (oracle/rsoracle.c) or, after
 * clshim_set_kernels(CLSHIM_KERNELS_RSCL) (or with CLSHIM_KERNELS=rscl in the
 * environment), with the reference's own rs.cl kernel compiled for the CPU
 * (oracle/ref/rscl.h), chosen by the kernel's source name (so the pass-2 name
 * swap of rs.c:506-507 is kept),
 * with the arguments rs.c set by index (the argument lists of rs.cl:374-1453
 * and the index enums of rs_priv.h:13-80) and the global offset and size of
 * the launch (rs.c:5342-5369).  Buffers and images live in host memory;
 * every enqueue completes before it returns, so events are placeholders.
 *
 * Device properties: one compute unit, work groups of up to 1024 items, a
 * preferred work-group multiple of 64 and 48 KB of local memory, so that
 * RS_revise_population rounds the background to multiples of 2048
 * (rs.c:2141) and RS_make_pulse_params plans its reductions as it would on
 * such a GPU (rs.c:1284-1386).
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "CL/cl.h"
#include "CL/cl_gl.h"
#include "rsoracle.h"
#include "rscl.h"
#include "clshim.h"

struct _cl_platform_id { int unused; };
struct _cl_device_id { int unused; };
struct _cl_context { int refs; };
struct _cl_command_queue { int refs; };
struct _cl_program { int refs; };
struct _cl_event { int refs; };

enum { MEM_BUFFER = 0, MEM_IMAGE = 1 };

struct _cl_mem {
    int kind;
    size_t size;          /* bytes */
    unsigned char *data;
    size_t nx, ny, nz;    /* image texels per axis (float4 texels) */
};

#define MAX_ARGS 24
enum { ARG_UNSET = 0, ARG_MEM, ARG_VALUE, ARG_LOCAL };

struct _cl_kernel {
    char name[64];
    struct {
        int kind;
        size_t size;
        cl_mem mem;
        unsigned char value[64];
    } arg[MAX_ARGS];
};

static struct _cl_platform_id g_platform;
static struct _cl_device_id g_device;

/* launch accounting, by kernel name */
#define MAX_NAMES 32
static struct {
    char name[64];
    unsigned long long launches;
} g_counts[MAX_NAMES];

static void count_launch(const char *name) {
    for (int i = 0; i < MAX_NAMES; i++) {
        if (g_counts[i].name[0] == '\0') {
            snprintf(g_counts[i].name, sizeof(g_counts[i].name), "%s", name);
        }
        if (strcmp(g_counts[i].name, name) == 0) {
            g_counts[i].launches++;
            return;
        }
    }
}

static char g_error[256];

static void (*g_hook)(const clshim_event *, void *);
static void *g_hook_user;

static void notify(int kind, cl_mem mem, size_t offset, size_t size, const void *ptr, cl_kernel k, size_t goff,
                   size_t gsize, size_t lsize) {
    if (g_hook == NULL) return;
    clshim_event e;
    memset(&e, 0, sizeof(e));
    e.kind = kind;
    e.mem = mem;
    e.offset = offset;
    e.size = size;
    e.ptr = ptr;
    e.kernel = k;
    e.name = k ? k->name : NULL;
    e.global_offset = goff;
    e.global_size = gsize;
    e.local_size = lsize;
    g_hook(&e, g_hook_user);
}

static void shim_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
    fprintf(stderr, "clshim: %s\n", g_error);
}

static cl_int set_ret(cl_int *ret, cl_int v) {
    if (ret) *ret = v;
    return v;
}

static cl_int put_info(const void *src, size_t n, size_t size, void *value, size_t *size_ret) {
    if (size_ret) *size_ret = n;
    if (value) {
        if (size < n) return CL_INVALID_VALUE;
        memcpy(value, src, n);
    }
    return CL_SUCCESS;
}

static cl_int put_string(const char *s, size_t size, void *value, size_t *size_ret) {
    return put_info(s, strlen(s) + 1, size, value, size_ret);
}

/* ---- platform and device ---- */

cl_int clGetPlatformIDs(cl_uint num_entries, cl_platform_id *platforms, cl_uint *num_platforms) {
    if (platforms && num_entries > 0) platforms[0] = &g_platform;
    if (num_platforms) *num_platforms = 1;
    return CL_SUCCESS;
}

cl_int clGetPlatformInfo(cl_platform_id platform, cl_platform_info name, size_t size, void *value,
                         size_t *size_ret) {
    (void)platform;
    switch (name) {
        case CL_PLATFORM_PROFILE: return put_string("FULL_PROFILE", size, value, size_ret);
        case CL_PLATFORM_VERSION: return put_string("OpenCL 1.2 (SimRadar CPU oracle shim)", size, value, size_ret);
        case CL_PLATFORM_NAME: return put_string("SimRadar CPU oracle shim", size, value, size_ret);
        case CL_PLATFORM_VENDOR: return put_string("simradar_gb300 test infrastructure", size, value, size_ret);
        case CL_PLATFORM_EXTENSIONS: return put_string("", size, value, size_ret);
        default: return CL_INVALID_VALUE;
    }
}

cl_int clGetDeviceIDs(cl_platform_id platform, cl_device_type type, cl_uint num_entries, cl_device_id *devices,
                      cl_uint *num_devices) {
    (void)platform;
    (void)type;
    if (devices && num_entries > 0) devices[0] = &g_device;
    if (num_devices) *num_devices = 1;
    return CL_SUCCESS;
}

cl_int clGetDeviceInfo(cl_device_id device, cl_device_info name, size_t size, void *value, size_t *size_ret) {
    (void)device;
    cl_uint u;
    cl_ulong ul;
    size_t sz;
    cl_device_type t;
    size_t sizes[3];
    switch (name) {
        case CL_DEVICE_TYPE: t = CL_DEVICE_TYPE_GPU; return put_info(&t, sizeof(t), size, value, size_ret);
        case CL_DEVICE_MAX_COMPUTE_UNITS: u = 1; return put_info(&u, sizeof(u), size, value, size_ret);
        case CL_DEVICE_MAX_WORK_ITEM_DIMENSIONS: u = 3; return put_info(&u, sizeof(u), size, value, size_ret);
        case CL_DEVICE_MAX_WORK_GROUP_SIZE: sz = 1024; return put_info(&sz, sizeof(sz), size, value, size_ret);
        case CL_DEVICE_MAX_WORK_ITEM_SIZES:
            sizes[0] = 1024; sizes[1] = 1024; sizes[2] = 64;
            return put_info(sizes, sizeof(sizes), size, value, size_ret);
        case CL_DEVICE_MAX_CLOCK_FREQUENCY: u = 1000; return put_info(&u, sizeof(u), size, value, size_ret);
        case CL_DEVICE_MAX_MEM_ALLOC_SIZE: ul = 16ull << 30; return put_info(&ul, sizeof(ul), size, value, size_ret);
        case CL_DEVICE_GLOBAL_MEM_SIZE: ul = 64ull << 30; return put_info(&ul, sizeof(ul), size, value, size_ret);
        case CL_DEVICE_MAX_CONSTANT_BUFFER_SIZE: ul = 64ull << 10; return put_info(&ul, sizeof(ul), size, value, size_ret);
        case CL_DEVICE_LOCAL_MEM_SIZE: ul = 48ull << 10; return put_info(&ul, sizeof(ul), size, value, size_ret);
        case CL_DEVICE_IMAGE2D_MAX_WIDTH:
        case CL_DEVICE_IMAGE2D_MAX_HEIGHT: sz = 16384; return put_info(&sz, sizeof(sz), size, value, size_ret);
        case CL_DEVICE_IMAGE3D_MAX_WIDTH:
        case CL_DEVICE_IMAGE3D_MAX_HEIGHT:
        case CL_DEVICE_IMAGE3D_MAX_DEPTH: sz = 2048; return put_info(&sz, sizeof(sz), size, value, size_ret);
        case CL_DEVICE_NAME: return put_string("CPU oracle (rs.cl restated in C)", size, value, size_ret);
        case CL_DEVICE_VENDOR: return put_string("simradar_gb300 test infrastructure", size, value, size_ret);
        case CL_DRIVER_VERSION: return put_string("1.0", size, value, size_ret);
        case CL_DEVICE_VERSION: return put_string("OpenCL 1.2", size, value, size_ret);
        default: return CL_INVALID_VALUE;
    }
}

/* ---- context, queue, program ---- */

cl_context clCreateContext(const cl_context_properties *properties, cl_uint num_devices, const cl_device_id *devices,
                           void (*pfn_notify)(const char *, const void *, size_t, void *), void *user_data,
                           cl_int *ret) {
    (void)properties; (void)num_devices; (void)devices; (void)pfn_notify; (void)user_data;
    cl_context c = (cl_context)calloc(1, sizeof(*c));
    set_ret(ret, c ? CL_SUCCESS : CL_OUT_OF_HOST_MEMORY);
    return c;
}

cl_int clReleaseContext(cl_context c) {
    free(c);
    return CL_SUCCESS;
}

cl_command_queue clCreateCommandQueue(cl_context context, cl_device_id device, cl_command_queue_properties props,
                                      cl_int *ret) {
    (void)context; (void)device; (void)props;
    cl_command_queue q = (cl_command_queue)calloc(1, sizeof(*q));
    set_ret(ret, q ? CL_SUCCESS : CL_OUT_OF_HOST_MEMORY);
    return q;
}

cl_int clReleaseCommandQueue(cl_command_queue q) {
    free(q);
    return CL_SUCCESS;
}

cl_program clCreateProgramWithSource(cl_context context, cl_uint count, const char **strings, const size_t *lengths,
                                     cl_int *ret) {
    (void)context; (void)count; (void)strings; (void)lengths;
    cl_program p = (cl_program)calloc(1, sizeof(*p));
    set_ret(ret, p ? CL_SUCCESS : CL_OUT_OF_HOST_MEMORY);
    return p;
}

/* The kernels are the oracle's, compiled with this library: nothing to build. */
cl_int clBuildProgram(cl_program program, cl_uint num_devices, const cl_device_id *devices, const char *options,
                      void (*pfn_notify)(cl_program, void *), void *user_data) {
    (void)num_devices; (void)devices; (void)options; (void)user_data;
    if (pfn_notify) pfn_notify(program, user_data);
    return CL_SUCCESS;
}

cl_int clGetProgramBuildInfo(cl_program program, cl_device_id device, cl_program_build_info name, size_t size,
                             void *value, size_t *size_ret) {
    (void)program; (void)device;
    if (name == CL_PROGRAM_BUILD_LOG) return put_string("", size, value, size_ret);
    return CL_INVALID_VALUE;
}

cl_int clReleaseProgram(cl_program p) {
    free(p);
    return CL_SUCCESS;
}

/* ---- kernels ---- */

static const char *const k_names[] = {
    "io", "dummy", "db_rcs", "bg_atts", "fp_atts", "el_atts", "db_atts", "scat_clr", "scat_sig_aux",
    "make_pulse_pass_1", "make_pulse_pass_2_group", "make_pulse_pass_2_local", "make_pulse_pass_2_range", "pop"};

cl_kernel clCreateKernel(cl_program program, const char *name, cl_int *ret) {
    (void)program;
    int known = 0;
    for (size_t i = 0; i < sizeof(k_names) / sizeof(k_names[0]); i++) {
        if (strcmp(name, k_names[i]) == 0) known = 1;
    }
    if (!known) {
        shim_error("no kernel named %s", name);
        set_ret(ret, CL_INVALID_KERNEL_NAME);
        return NULL;
    }
    cl_kernel k = (cl_kernel)calloc(1, sizeof(*k));
    if (k == NULL) {
        set_ret(ret, CL_OUT_OF_HOST_MEMORY);
        return NULL;
    }
    snprintf(k->name, sizeof(k->name), "%s", name);
    set_ret(ret, CL_SUCCESS);
    return k;
}

cl_int clReleaseKernel(cl_kernel k) {
    free(k);
    return CL_SUCCESS;
}

/* Memory arguments are told from values by the pointer they point at: a
 * cl_mem of this library (rs.c passes &C->scat_pos and the like). */
#define MAX_MEMS 4096
static cl_mem g_mems[MAX_MEMS];

static int is_mem(cl_mem m) {
    if (m == NULL) return 0;
    for (int i = 0; i < MAX_MEMS; i++) {
        if (g_mems[i] == m) return 1;
    }
    return 0;
}

cl_int clSetKernelArg(cl_kernel k, cl_uint index, size_t size, const void *value) {
    if (k == NULL) return CL_INVALID_KERNEL;
    if (index >= MAX_ARGS) return CL_INVALID_ARG_INDEX;
    if (value == NULL) {
        /* __local memory of `size` bytes (the pass-1 / pass-2 scratch) */
        k->arg[index].kind = ARG_LOCAL;
        k->arg[index].size = size;
        return CL_SUCCESS;
    }
    /* a NULL cl_mem is a NULL pointer argument (the debris-flux table of
     * db_atts before any is set, rs.c:5360) */
    if (size == sizeof(cl_mem) && (*(const cl_mem *)value == NULL || is_mem(*(const cl_mem *)value))) {
        k->arg[index].kind = ARG_MEM;
        k->arg[index].mem = *(const cl_mem *)value;
        k->arg[index].size = size;
        return CL_SUCCESS;
    }
    if (size > sizeof(k->arg[index].value)) return CL_INVALID_ARG_SIZE;
    k->arg[index].kind = ARG_VALUE;
    k->arg[index].size = size;
    memcpy(k->arg[index].value, value, size);
    return CL_SUCCESS;
}

cl_int clGetKernelWorkGroupInfo(cl_kernel k, cl_device_id device, cl_kernel_work_group_info name, size_t size,
                                void *value, size_t *size_ret) {
    (void)k; (void)device;
    size_t v;
    if (name == CL_KERNEL_PREFERRED_WORK_GROUP_SIZE_MULTIPLE) {
        v = 64;
    } else if (name == CL_KERNEL_WORK_GROUP_SIZE) {
        v = 1024;
    } else {
        return CL_INVALID_VALUE;
    }
    return put_info(&v, sizeof(v), size, value, size_ret);
}

/* ---- memory objects ---- */

static cl_mem new_mem(int kind, size_t size, const void *host, cl_mem_flags flags, cl_int *ret) {
    cl_mem m = (cl_mem)calloc(1, sizeof(*m));
    if (m == NULL) {
        set_ret(ret, CL_OUT_OF_HOST_MEMORY);
        return NULL;
    }
    m->kind = kind;
    m->size = size;
    m->data = (unsigned char *)calloc(size ? size : 1, 1);
    if (m->data == NULL) {
        free(m);
        set_ret(ret, CL_MEM_OBJECT_ALLOCATION_FAILURE);
        return NULL;
    }
    if (host && (flags & (CL_MEM_COPY_HOST_PTR | CL_MEM_USE_HOST_PTR))) memcpy(m->data, host, size);
    int slot = -1;
    for (int i = 0; i < MAX_MEMS; i++) {
        if (g_mems[i] == NULL) {
            slot = i;
            break;
        }
    }
    if (slot < 0) {
        free(m->data);
        free(m);
        shim_error("more than %d memory objects", MAX_MEMS);
        set_ret(ret, CL_OUT_OF_HOST_MEMORY);
        return NULL;
    }
    g_mems[slot] = m;
    set_ret(ret, CL_SUCCESS);
    return m;
}

cl_mem clCreateBuffer(cl_context context, cl_mem_flags flags, size_t size, void *host, cl_int *ret) {
    (void)context;
    return new_mem(MEM_BUFFER, size, host, flags, ret);
}

static cl_mem new_image(cl_mem_flags flags, const cl_image_format *fmt, size_t nx, size_t ny, size_t nz,
                        void *host, cl_int *ret) {
    if (fmt == NULL || fmt->image_channel_order != CL_RGBA || fmt->image_channel_data_type != CL_FLOAT) {
        shim_error("images are CL_RGBA / CL_FLOAT only");
        set_ret(ret, CL_INVALID_VALUE);
        return NULL;
    }
    if (nx == 0 || ny == 0 || nz == 0) {
        set_ret(ret, CL_INVALID_IMAGE_SIZE);
        return NULL;
    }
    cl_mem m = new_mem(MEM_IMAGE, nx * ny * nz * 16, host, flags, ret);
    if (m) {
        m->nx = nx;
        m->ny = ny;
        m->nz = nz;
    }
    return m;
}

cl_mem clCreateImage(cl_context context, cl_mem_flags flags, const cl_image_format *fmt, const cl_image_desc *desc,
                     void *host, cl_int *ret) {
    (void)context;
    if (desc == NULL) {
        set_ret(ret, CL_INVALID_VALUE);
        return NULL;
    }
    if (desc->image_type == CL_MEM_OBJECT_IMAGE2D) {
        return new_image(flags, fmt, desc->image_width, desc->image_height, 1, host, ret);
    }
    if (desc->image_type == CL_MEM_OBJECT_IMAGE3D) {
        return new_image(flags, fmt, desc->image_width, desc->image_height, desc->image_depth, host, ret);
    }
    set_ret(ret, CL_INVALID_VALUE);
    return NULL;
}

cl_mem clCreateImage2D(cl_context context, cl_mem_flags flags, const cl_image_format *fmt, size_t w, size_t h,
                       size_t row_pitch, void *host, cl_int *ret) {
    (void)context; (void)row_pitch;
    return new_image(flags, fmt, w, h, 1, host, ret);
}

cl_mem clCreateImage3D(cl_context context, cl_mem_flags flags, const cl_image_format *fmt, size_t w, size_t h,
                       size_t d, size_t row_pitch, size_t slice_pitch, void *host, cl_int *ret) {
    (void)context; (void)row_pitch; (void)slice_pitch;
    return new_image(flags, fmt, w, h, d, host, ret);
}

cl_mem clCreateFromGLBuffer(cl_context context, cl_mem_flags flags, cl_GLuint bufobj, cl_int *ret) {
    (void)context; (void)flags; (void)bufobj;
    shim_error("no OpenGL in this build");
    set_ret(ret, CL_INVALID_GL_OBJECT);
    return NULL;
}

cl_int clReleaseMemObject(cl_mem m) {
    if (m == NULL) return CL_INVALID_MEM_OBJECT;
    for (int i = 0; i < MAX_MEMS; i++) {
        if (g_mems[i] == m) g_mems[i] = NULL;
    }
    free(m->data);
    free(m);
    return CL_SUCCESS;
}

/* ---- transfers (complete on return) ---- */

static cl_event new_event(void) { return (cl_event)calloc(1, sizeof(struct _cl_event)); }

cl_int clEnqueueWriteBuffer(cl_command_queue q, cl_mem b, cl_bool blocking, size_t offset, size_t size,
                            const void *ptr, cl_uint nw, const cl_event *wl, cl_event *ev) {
    (void)q; (void)blocking; (void)nw; (void)wl;
    if (!is_mem(b) || offset + size > b->size) return CL_INVALID_VALUE;
    notify(CLSHIM_WRITE_BUFFER, b, offset, size, ptr, NULL, 0, 0, 0);
    memcpy(b->data + offset, ptr, size);
    if (ev) *ev = new_event();
    return CL_SUCCESS;
}

cl_int clEnqueueReadBuffer(cl_command_queue q, cl_mem b, cl_bool blocking, size_t offset, size_t size, void *ptr,
                           cl_uint nw, const cl_event *wl, cl_event *ev) {
    (void)q; (void)blocking; (void)nw; (void)wl;
    if (!is_mem(b) || offset + size > b->size) return CL_INVALID_VALUE;
    memcpy(ptr, b->data + offset, size);
    if (ev) *ev = new_event();
    return CL_SUCCESS;
}

cl_int clEnqueueWriteImage(cl_command_queue q, cl_mem im, cl_bool blocking, const size_t *origin,
                           const size_t *region, size_t row_pitch, size_t slice_pitch, const void *ptr, cl_uint nw,
                           const cl_event *wl, cl_event *ev) {
    (void)q; (void)blocking; (void)nw; (void)wl;
    if (!is_mem(im) || im->kind != MEM_IMAGE) return CL_INVALID_MEM_OBJECT;
    if (origin[0] + region[0] > im->nx || origin[1] + region[1] > im->ny || origin[2] + region[2] > im->nz) {
        return CL_INVALID_VALUE;
    }
    notify(CLSHIM_WRITE_IMAGE, im, 0, region[0] * region[1] * region[2] * 16, ptr, NULL, 0, 0, 0);
    const size_t rp = row_pitch ? row_pitch : region[0] * 16;
    const size_t sp = slice_pitch ? slice_pitch : rp * region[1];
    for (size_t z = 0; z < region[2]; z++) {
        for (size_t y = 0; y < region[1]; y++) {
            const unsigned char *src = (const unsigned char *)ptr + z * sp + y * rp;
            unsigned char *dst = im->data + (((origin[2] + z) * im->ny + origin[1] + y) * im->nx + origin[0]) * 16;
            memcpy(dst, src, region[0] * 16);
        }
    }
    if (ev) *ev = new_event();
    return CL_SUCCESS;
}

/* ---- launches ---- */

static int need(cl_kernel k, cl_uint i, int kind) {
    if (k->arg[i].kind != kind) {
        shim_error("%s: argument %u not set as %s", k->name, i,
                   kind == ARG_MEM ? "a memory object" : (kind == ARG_VALUE ? "a value" : "local memory"));
        return 0;
    }
    return 1;
}

static void *buf(cl_kernel k, cl_uint i) { return k->arg[i].mem ? k->arg[i].mem->data : NULL; }
static size_t buf_n16(cl_kernel k, cl_uint i) { return k->arg[i].mem ? k->arg[i].mem->size / 16 : 0; }
static const float *val_f(cl_kernel k, cl_uint i) { return (const float *)k->arg[i].value; }
static cl_uint val_u(cl_kernel k, cl_uint i) { return *(const cl_uint *)k->arg[i].value; }

static or_image img(cl_kernel k, cl_uint i) {
    or_image r;
    cl_mem m = k->arg[i].mem;
    if (m == NULL) {
        memset(&r, 0, sizeof(r));
        return r;
    }
    r.data = (const of4 *)m->data;
    r.nx = (int)m->nx;
    r.ny = (int)m->ny;
    r.nz = (int)m->nz;
    return r;
}

/* argument kinds per kernel, in the order of its rs.cl parameter list:
 * m memory object (buffer or image), v value, l local memory */
static const struct {
    const char *name;
    const char *kinds;
} k_sigs[] = {
    {"bg_atts", "mmmmmmvmvv"},              /* rs.cl:533-542 */
    {"el_atts", "mmmmmmvmvv"},              /* rs.cl:653-662 */
    {"fp_atts", "mmmmmmvmvv"},              /* rs.cl:590-599 */
    {"db_atts", "mmmmmmmmvmmvmmvmvv"},      /* rs.cl:744-761 */
    {"db_rcs", "mmmmmvv"},                  /* rs.cl:909-915 */
    {"scat_sig_aux", "mmmmmvv"},            /* rs.cl:1050-1056 */
    {"make_pulse_pass_1", "mmmlmvvvvvv"},   /* rs.cl:1125-1135 */
    {"make_pulse_pass_2_local", "mmlvv"},   /* rs.cl:1304-1308 */
    {"make_pulse_pass_2_range", "mmlvv"},   /* rs.cl:1341-1345 */
    {"make_pulse_pass_2_group", "mmlvv"},   /* rs.cl:1362-1366 */
    {"pop", "mmmv"},                        /* rs.cl:1444 */
};

static int check_args(cl_kernel k) {
    for (size_t s = 0; s < sizeof(k_sigs) / sizeof(k_sigs[0]); s++) {
        if (strcmp(k_sigs[s].name, k->name) != 0) continue;
        const char *kinds = k_sigs[s].kinds;
        for (cl_uint i = 0; kinds[i]; i++) {
            const int want = kinds[i] == 'm' ? ARG_MEM : (kinds[i] == 'v' ? ARG_VALUE : ARG_LOCAL);
            if (!need(k, i, want)) return 0;
        }
        return 1;
    }
    shim_error("kernel %s is not run by this device", k->name);
    return 0;
}

/* which kernels the device runs: the oracle's restatement or the
 * reference's rs.cl (CLSHIM_KERNELS=rscl selects the latter at start) */
static int g_kernels = -1;

void clshim_set_kernels(int which) { g_kernels = which; }

static int kernels_rscl(void) {
    if (g_kernels < 0) {
        const char *e = getenv("CLSHIM_KERNELS");
        g_kernels = (e != NULL && !strcmp(e, "rscl")) ? CLSHIM_KERNELS_RSCL : CLSHIM_KERNELS_ORACLE;
    }
    return g_kernels == CLSHIM_KERNELS_RSCL;
}

cl_int clEnqueueNDRangeKernel(cl_command_queue q, cl_kernel k, cl_uint dim, const size_t *goff, const size_t *gsize,
                              const size_t *lsize, cl_uint nw, const cl_event *wl, cl_event *ev) {
    (void)q; (void)nw; (void)wl;
    if (k == NULL) return CL_INVALID_KERNEL;
    if (dim != 1) return CL_INVALID_WORK_DIMENSION;
    if (!check_args(k)) return CL_INVALID_KERNEL;
    const size_t origin = goff ? goff[0] : 0;
    const size_t count = gsize[0];
    const size_t local = lsize ? lsize[0] : 0;
    const char *n = k->name;
    notify(CLSHIM_LAUNCH, NULL, 0, 0, NULL, k, origin, count, local);
    const int ref = kernels_rscl();
    if (!strcmp(n, "bg_atts") || !strcmp(n, "el_atts")) {
        if (origin + count > buf_n16(k, 0)) return CL_INVALID_GLOBAL_OFFSET;
        void (*f)(of4 *, of4 *, of4 *, ou4 *, or_image, const float *, const of4 *, const float *, const float *,
                  size_t, size_t) = n[0] == 'b' ? (ref ? rscl_bg_atts : or_bg_atts) : (ref ? rscl_el_atts : or_el_atts);
        f((of4 *)buf(k, 0), (of4 *)buf(k, 1), (of4 *)buf(k, 2), (ou4 *)buf(k, 3), img(k, 4), val_f(k, 6),
          (const of4 *)buf(k, 7), val_f(k, 8), val_f(k, 9), origin, count);
    } else if (!strcmp(n, "fp_atts")) {
        if (origin + count > buf_n16(k, 0)) return CL_INVALID_GLOBAL_OFFSET;
        (ref ? rscl_fp_atts : or_fp_atts)((of4 *)buf(k, 0), (of4 *)buf(k, 1), (of4 *)buf(k, 2), img(k, 4), img(k, 5),
                                          val_f(k, 6), val_f(k, 9), origin, count);
    } else if (!strcmp(n, "db_atts")) {
        if (origin + count > buf_n16(k, 0)) return CL_INVALID_GLOBAL_OFFSET;
        (ref ? rscl_db_atts : or_db_atts)((of4 *)buf(k, 0), (of4 *)buf(k, 1), (of4 *)buf(k, 2), (of4 *)buf(k, 3),
                                          (of4 *)buf(k, 4), (ou4 *)buf(k, 5), img(k, 6), val_f(k, 8), img(k, 9),
                                          img(k, 10), val_f(k, 11), img(k, 12), img(k, 13), val_f(k, 14),
                                          (const float *)buf(k, 15), val_f(k, 16), val_f(k, 17), origin, count);
    } else if (!strcmp(n, "db_rcs")) {
        if (origin + count > buf_n16(k, 0)) return CL_INVALID_GLOBAL_OFFSET;
        (ref ? rscl_db_rcs : or_db_rcs)((const of4 *)buf(k, 0), (const of4 *)buf(k, 1), (of4 *)buf(k, 2), img(k, 3),
                                        img(k, 4), val_f(k, 5), val_f(k, 6), origin, count);
    } else if (!strcmp(n, "scat_sig_aux")) {
        if (origin != 0 || count > buf_n16(k, 0)) return CL_INVALID_GLOBAL_OFFSET;
        (ref ? rscl_scat_sig_aux : or_scat_sig_aux)((of4 *)buf(k, 0), (of4 *)buf(k, 1), (const of4 *)buf(k, 2),
                                                    (const of4 *)buf(k, 3), (const float *)buf(k, 4), val_f(k, 5),
                                                    val_f(k, 6), count);
    } else if (!strcmp(n, "make_pulse_pass_1")) {
        const cl_uint range_count = val_u(k, 8), group_count = val_u(k, 9), items = val_u(k, 10);
        if (local == 0 || (size_t)group_count * range_count > buf_n16(k, 0)) return CL_INVALID_VALUE;
        (ref ? rscl_make_pulse_pass_1 : or_make_pulse_pass_1)(
            (of4 *)buf(k, 0), (const of4 *)buf(k, 1), (const of4 *)buf(k, 2), buf_n16(k, 1), (const float *)buf(k, 4),
            val_f(k, 5), *val_f(k, 6), *val_f(k, 7), range_count, group_count, items, (uint32_t)local);
    } else if (!strncmp(n, "make_pulse_pass_2_", 18)) {
        /* Pass 2 writes out[get_global_id(0)] for every work item, and its
         * global size is the launch plan's (rs.c:1355-1382), which can exceed
         * the range_count entries of the pulse buffer: the body runs into a
         * scratch array of the launch's size and the buffer gets its part. */
        const size_t nout = buf_n16(k, 0) > count ? buf_n16(k, 0) : count;
        of4 *tmp = (of4 *)calloc(nout ? nout : 1, sizeof(of4));
        if (tmp == NULL) return CL_OUT_OF_HOST_MEMORY;
        const of4 *in = (const of4 *)buf(k, 1);
        const size_t in_n = buf_n16(k, 1);
        if (!strcmp(n, "make_pulse_pass_2_local")) {
            if (ref) {
                rscl_make_pulse_pass_2_local(tmp, in, in_n, val_u(k, 3), val_u(k, 4), count, local);
            } else {
                or_make_pulse_pass_2_local_body(tmp, in, in_n, val_u(k, 3), val_u(k, 4), count, local);
            }
        } else if (!strcmp(n, "make_pulse_pass_2_range")) {
            if (ref) {
                rscl_make_pulse_pass_2_range(tmp, in, in_n, val_u(k, 3), val_u(k, 4), count, local);
            } else {
                or_make_pulse_pass_2_range_body(tmp, in, in_n, val_u(k, 3), val_u(k, 4), count);
            }
        } else {
            if (ref) {
                rscl_make_pulse_pass_2_group(tmp, in, in_n, val_u(k, 3), val_u(k, 4), count, local);
            } else {
                or_make_pulse_pass_2_group_body(tmp, in, in_n, val_u(k, 3), local);
            }
        }
        memcpy(buf(k, 0), tmp, buf_n16(k, 0) * sizeof(of4));
        free(tmp);
    } else if (!strcmp(n, "pop")) {
        if (origin != 0 || count > buf_n16(k, 0)) return CL_INVALID_GLOBAL_OFFSET;
        (ref ? rscl_pop : or_pop)((of4 *)buf(k, 0), (of4 *)buf(k, 1), (of4 *)buf(k, 2), val_f(k, 3), count);
    } else {
        shim_error("kernel %s is not run by this device", n);
        return CL_INVALID_KERNEL;
    }
    count_launch(n);
    if (ev) *ev = new_event();
    return CL_SUCCESS;
}

cl_int clFlush(cl_command_queue q) {
    (void)q;
    return CL_SUCCESS;
}

cl_int clFinish(cl_command_queue q) {
    (void)q;
    return CL_SUCCESS;
}

cl_int clWaitForEvents(cl_uint n, const cl_event *list) {
    (void)n; (void)list;
    return CL_SUCCESS;
}

cl_int clReleaseEvent(cl_event e) {
    free(e);
    return CL_SUCCESS;
}

/* ---- inspection (clshim.h) ---- */

const void *clshim_mem_data(cl_mem m, size_t *bytes, size_t dims[3]) {
    if (!is_mem(m)) return NULL;
    if (bytes) *bytes = m->size;
    if (dims) {
        dims[0] = m->kind == MEM_IMAGE ? m->nx : m->size / 16;
        dims[1] = m->kind == MEM_IMAGE ? m->ny : 1;
        dims[2] = m->kind == MEM_IMAGE ? m->nz : 1;
    }
    return m->data;
}

unsigned long long clshim_launches(const char *name) {
    for (int i = 0; i < MAX_NAMES; i++) {
        if (strcmp(g_counts[i].name, name) == 0) return g_counts[i].launches;
    }
    return 0;
}

const char *clshim_last_error(void) { return g_error; }

int clshim_kernel_arg(cl_kernel k, unsigned index, void *out, size_t size) {
    if (k == NULL || index >= MAX_ARGS) return -1;
    if (k->arg[index].kind == ARG_MEM) {
        if (size != sizeof(cl_mem)) return -1;
        memcpy(out, &k->arg[index].mem, sizeof(cl_mem));
        return 0;
    }
    if (k->arg[index].kind != ARG_VALUE || size > k->arg[index].size) return -1;
    memcpy(out, k->arg[index].value, size);
    return 0;
}

void clshim_set_hook(void (*hook)(const clshim_event *, void *), void *user) {
    g_hook = hook;
    g_hook_user = user;
}
