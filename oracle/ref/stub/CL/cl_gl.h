/*
 * The one OpenCL / OpenGL interop entry point the reference host (rs.c)
 * names, declared for this project from the public Khronos API.  There is no
 * graphics stack in this build: the CL shim's definition returns
 * CL_INVALID_GL_OBJECT, and rs.c only calls it when a GUI shares its vertex
 * buffers (RS_share_mem_with_vbo), which never happens here.
 */
#ifndef SIMRADAR_CLSHIM_CL_GL_H
#define SIMRADAR_CLSHIM_CL_GL_H

#include "cl.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned int cl_GLuint;

cl_mem clCreateFromGLBuffer(cl_context context, cl_mem_flags flags, cl_GLuint bufobj, cl_int *errcode_ret);

#ifdef __cplusplus
}
#endif

#endif
