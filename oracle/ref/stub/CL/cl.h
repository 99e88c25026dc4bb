/*
 * A minimal OpenCL 1.2 host API declaration, written for this project from
 * the public Khronos API names, covering only the subset the reference host
 * (rs.c) uses.  There is no OpenCL SDK in this build's image: this header lets
 * the unmodified rs.c compile, and oracle/ref/clshim.c implements every entry
 * point declared here on the CPU oracle (a device that runs the restated
 * rs.cl kernels).  Test infrastructure only.
 *
 * The scalar and vector types follow the Khronos layout (cl_float4 is four
 * floats addressable as .s[i], .x .. .w, .s0 .. .s3, .lo / .hi), so rs.c's
 * host structures keep their size and field offsets.
 */
#ifndef SIMRADAR_CLSHIM_CL_H
#define SIMRADAR_CLSHIM_CL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CL_VERSION_1_0 1
#define CL_VERSION_1_1 1
#define CL_VERSION_1_2 1

#define CL_API_ENTRY
#define CL_API_CALL
#define CL_CALLBACK
#define CL_ALIGNED(n) __attribute__((aligned(n)))

typedef int8_t cl_char;
typedef uint8_t cl_uchar;
typedef int16_t cl_short;
typedef uint16_t cl_ushort;
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef int64_t cl_long;
typedef uint64_t cl_ulong;
typedef float cl_float;
typedef double cl_double;
typedef cl_uint cl_bool;
typedef cl_ulong cl_bitfield;

/* vector types: unions of an array and named lanes (anonymous members) */
#define CLSHIM_VEC2(T, N)                                                      \
    typedef union {                                                            \
        T CL_ALIGNED(2 * sizeof(T)) s[2];                                      \
        struct { T x, y; };                                                    \
        struct { T s0, s1; };                                                  \
        struct { T lo, hi; };                                                  \
    } N;
#define CLSHIM_VEC4(T, T2, N)                                                  \
    typedef union {                                                            \
        T CL_ALIGNED(4 * sizeof(T)) s[4];                                      \
        struct { T x, y, z, w; };                                              \
        struct { T s0, s1, s2, s3; };                                          \
        struct { T2 lo, hi; };                                                 \
    } N;
CLSHIM_VEC2(cl_float, cl_float2)
CLSHIM_VEC2(cl_double, cl_double2)
CLSHIM_VEC2(cl_uint, cl_uint2)
CLSHIM_VEC2(cl_int, cl_int2)
CLSHIM_VEC4(cl_float, cl_float2, cl_float4)
CLSHIM_VEC4(cl_double, cl_double2, cl_double4)
CLSHIM_VEC4(cl_uint, cl_uint2, cl_uint4)
CLSHIM_VEC4(cl_int, cl_int2, cl_int4)
typedef union {
    cl_float CL_ALIGNED(32) s[8];
    struct { cl_float x, y, z, w; };
    struct { cl_float s0, s1, s2, s3, s4, s5, s6, s7; };
    struct { cl_float4 lo, hi; };
} cl_float8;
typedef union {
    cl_float CL_ALIGNED(64) s[16];
    struct { cl_float x, y, z, w; };
    struct { cl_float s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sA, sB, sC, sD, sE, sF; };
    struct { cl_float8 lo, hi; };
} cl_float16;
#undef CLSHIM_VEC2
#undef CLSHIM_VEC4

typedef struct _cl_platform_id *cl_platform_id;
typedef struct _cl_device_id *cl_device_id;
typedef struct _cl_context *cl_context;
typedef struct _cl_command_queue *cl_command_queue;
typedef struct _cl_mem *cl_mem;
typedef struct _cl_program *cl_program;
typedef struct _cl_kernel *cl_kernel;
typedef struct _cl_event *cl_event;
typedef struct _cl_sampler *cl_sampler;

typedef cl_bitfield cl_device_type;
typedef cl_uint cl_platform_info;
typedef cl_uint cl_device_info;
typedef cl_bitfield cl_command_queue_properties;
typedef intptr_t cl_context_properties;
typedef cl_uint cl_context_info;
typedef cl_bitfield cl_mem_flags;
typedef cl_uint cl_mem_object_type;
typedef cl_uint cl_channel_order;
typedef cl_uint cl_channel_type;
typedef cl_uint cl_program_build_info;
typedef cl_uint cl_kernel_work_group_info;
typedef cl_bitfield cl_map_flags;

typedef struct {
    cl_channel_order image_channel_order;
    cl_channel_type image_channel_data_type;
} cl_image_format;

typedef struct {
    cl_mem_object_type image_type;
    size_t image_width;
    size_t image_height;
    size_t image_depth;
    size_t image_array_size;
    size_t image_row_pitch;
    size_t image_slice_pitch;
    cl_uint num_mip_levels;
    cl_uint num_samples;
    cl_mem buffer;
} cl_image_desc;

/* status codes */
#define CL_SUCCESS 0
#define CL_DEVICE_NOT_FOUND -1
#define CL_MEM_OBJECT_ALLOCATION_FAILURE -4
#define CL_OUT_OF_HOST_MEMORY -6
#define CL_BUILD_PROGRAM_FAILURE -11
#define CL_INVALID_VALUE -30
#define CL_INVALID_DEVICE -33
#define CL_INVALID_CONTEXT -34
#define CL_INVALID_MEM_OBJECT -38
#define CL_INVALID_IMAGE_SIZE -40
#define CL_INVALID_KERNEL_NAME -46
#define CL_INVALID_KERNEL -48
#define CL_INVALID_ARG_INDEX -49
#define CL_INVALID_ARG_VALUE -50
#define CL_INVALID_ARG_SIZE -51
#define CL_INVALID_WORK_DIMENSION -53
#define CL_INVALID_GLOBAL_OFFSET -56
#define CL_INVALID_OPERATION -59
#define CL_INVALID_GL_OBJECT -60

#define CL_FALSE 0
#define CL_TRUE 1

/* device types */
#define CL_DEVICE_TYPE_DEFAULT (1 << 0)
#define CL_DEVICE_TYPE_CPU (1 << 1)
#define CL_DEVICE_TYPE_GPU (1 << 2)
#define CL_DEVICE_TYPE_ACCELERATOR (1 << 3)
#define CL_DEVICE_TYPE_ALL 0xFFFFFFFF

/* platform info */
#define CL_PLATFORM_PROFILE 0x0900
#define CL_PLATFORM_VERSION 0x0901
#define CL_PLATFORM_NAME 0x0902
#define CL_PLATFORM_VENDOR 0x0903
#define CL_PLATFORM_EXTENSIONS 0x0904

/* device info */
#define CL_DEVICE_TYPE 0x1000
#define CL_DEVICE_MAX_COMPUTE_UNITS 0x1002
#define CL_DEVICE_MAX_WORK_ITEM_DIMENSIONS 0x1003
#define CL_DEVICE_MAX_WORK_GROUP_SIZE 0x1004
#define CL_DEVICE_MAX_WORK_ITEM_SIZES 0x1005
#define CL_DEVICE_MAX_CLOCK_FREQUENCY 0x100C
#define CL_DEVICE_MAX_MEM_ALLOC_SIZE 0x1010
#define CL_DEVICE_IMAGE2D_MAX_WIDTH 0x1011
#define CL_DEVICE_IMAGE2D_MAX_HEIGHT 0x1012
#define CL_DEVICE_IMAGE3D_MAX_WIDTH 0x1013
#define CL_DEVICE_IMAGE3D_MAX_HEIGHT 0x1014
#define CL_DEVICE_IMAGE3D_MAX_DEPTH 0x1015
#define CL_DEVICE_GLOBAL_MEM_SIZE 0x101F
#define CL_DEVICE_MAX_CONSTANT_BUFFER_SIZE 0x1020
#define CL_DEVICE_LOCAL_MEM_SIZE 0x1023
#define CL_DEVICE_NAME 0x102B
#define CL_DEVICE_VENDOR 0x102C
#define CL_DRIVER_VERSION 0x102D
#define CL_DEVICE_VERSION 0x102F

/* memory flags */
#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)
#define CL_MEM_USE_HOST_PTR (1 << 3)
#define CL_MEM_ALLOC_HOST_PTR (1 << 4)
#define CL_MEM_COPY_HOST_PTR (1 << 5)

/* image formats and types */
#define CL_RGBA 0x10B5
#define CL_FLOAT 0x10DE
#define CL_MEM_OBJECT_BUFFER 0x10F0
#define CL_MEM_OBJECT_IMAGE2D 0x10F1
#define CL_MEM_OBJECT_IMAGE3D 0x10F2

/* program and kernel queries */
#define CL_PROGRAM_BUILD_LOG 0x1183
#define CL_KERNEL_WORK_GROUP_SIZE 0x11B0
#define CL_KERNEL_PREFERRED_WORK_GROUP_SIZE_MULTIPLE 0x11B3

cl_int clGetPlatformIDs(cl_uint num_entries, cl_platform_id *platforms, cl_uint *num_platforms);
cl_int clGetPlatformInfo(cl_platform_id platform, cl_platform_info param_name, size_t param_value_size,
                         void *param_value, size_t *param_value_size_ret);
cl_int clGetDeviceIDs(cl_platform_id platform, cl_device_type device_type, cl_uint num_entries,
                      cl_device_id *devices, cl_uint *num_devices);
cl_int clGetDeviceInfo(cl_device_id device, cl_device_info param_name, size_t param_value_size, void *param_value,
                       size_t *param_value_size_ret);
cl_context clCreateContext(const cl_context_properties *properties, cl_uint num_devices, const cl_device_id *devices,
                           void (*pfn_notify)(const char *, const void *, size_t, void *), void *user_data,
                           cl_int *errcode_ret);
cl_int clReleaseContext(cl_context context);
cl_command_queue clCreateCommandQueue(cl_context context, cl_device_id device,
                                      cl_command_queue_properties properties, cl_int *errcode_ret);
cl_int clReleaseCommandQueue(cl_command_queue command_queue);
cl_program clCreateProgramWithSource(cl_context context, cl_uint count, const char **strings, const size_t *lengths,
                                     cl_int *errcode_ret);
cl_int clBuildProgram(cl_program program, cl_uint num_devices, const cl_device_id *device_list, const char *options,
                      void (*pfn_notify)(cl_program, void *), void *user_data);
cl_int clGetProgramBuildInfo(cl_program program, cl_device_id device, cl_program_build_info param_name,
                             size_t param_value_size, void *param_value, size_t *param_value_size_ret);
cl_int clReleaseProgram(cl_program program);
cl_kernel clCreateKernel(cl_program program, const char *kernel_name, cl_int *errcode_ret);
cl_int clReleaseKernel(cl_kernel kernel);
cl_int clSetKernelArg(cl_kernel kernel, cl_uint arg_index, size_t arg_size, const void *arg_value);
cl_int clGetKernelWorkGroupInfo(cl_kernel kernel, cl_device_id device, cl_kernel_work_group_info param_name,
                                size_t param_value_size, void *param_value, size_t *param_value_size_ret);
cl_mem clCreateBuffer(cl_context context, cl_mem_flags flags, size_t size, void *host_ptr, cl_int *errcode_ret);
cl_mem clCreateImage(cl_context context, cl_mem_flags flags, const cl_image_format *image_format,
                     const cl_image_desc *image_desc, void *host_ptr, cl_int *errcode_ret);
cl_mem clCreateImage2D(cl_context context, cl_mem_flags flags, const cl_image_format *image_format,
                       size_t image_width, size_t image_height, size_t image_row_pitch, void *host_ptr,
                       cl_int *errcode_ret);
cl_mem clCreateImage3D(cl_context context, cl_mem_flags flags, const cl_image_format *image_format,
                       size_t image_width, size_t image_height, size_t image_depth, size_t image_row_pitch,
                       size_t image_slice_pitch, void *host_ptr, cl_int *errcode_ret);
cl_int clReleaseMemObject(cl_mem memobj);
cl_int clEnqueueWriteBuffer(cl_command_queue command_queue, cl_mem buffer, cl_bool blocking_write, size_t offset,
                            size_t size, const void *ptr, cl_uint num_events_in_wait_list,
                            const cl_event *event_wait_list, cl_event *event);
cl_int clEnqueueReadBuffer(cl_command_queue command_queue, cl_mem buffer, cl_bool blocking_read, size_t offset,
                           size_t size, void *ptr, cl_uint num_events_in_wait_list, const cl_event *event_wait_list,
                           cl_event *event);
cl_int clEnqueueWriteImage(cl_command_queue command_queue, cl_mem image, cl_bool blocking_write,
                           const size_t *origin, const size_t *region, size_t input_row_pitch,
                           size_t input_slice_pitch, const void *ptr, cl_uint num_events_in_wait_list,
                           const cl_event *event_wait_list, cl_event *event);
cl_int clEnqueueNDRangeKernel(cl_command_queue command_queue, cl_kernel kernel, cl_uint work_dim,
                              const size_t *global_work_offset, const size_t *global_work_size,
                              const size_t *local_work_size, cl_uint num_events_in_wait_list,
                              const cl_event *event_wait_list, cl_event *event);
cl_int clFlush(cl_command_queue command_queue);
cl_int clFinish(cl_command_queue command_queue);
cl_int clWaitForEvents(cl_uint num_events, const cl_event *event_list);
cl_int clReleaseEvent(cl_event event);

#ifdef __cplusplus
}
#endif

#endif
