/*
 * cl_types/CL/cl.h - the OpenCL 1.2 host types and constants (as the public
 * Khronos specification names them) that the reference's include/lib_icl.h
 * and src/abms.c refer to. Building abms.c over icl_sampo.cpp needs no
 * OpenCL platform or headers: this file stands in for them.
 */
#ifndef SAMPO_CL_TYPES_H
#define SAMPO_CL_TYPES_H
#include <stddef.h>
#include <stdint.h>

typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint64_t cl_ulong;
typedef float cl_float;
typedef cl_uint cl_bool;
typedef cl_ulong cl_bitfield;
typedef cl_bitfield cl_device_type;
typedef cl_bitfield cl_mem_flags;
typedef cl_bitfield cl_map_flags;
typedef cl_bitfield cl_device_fp_config;
typedef cl_uint cl_device_mem_cache_type;
typedef cl_uint cl_device_local_mem_type;

typedef struct _cl_device_id* cl_device_id;
typedef struct _cl_context* cl_context;
typedef struct _cl_command_queue* cl_command_queue;
typedef struct _cl_mem* cl_mem;
typedef struct _cl_kernel* cl_kernel;
typedef struct _cl_event* cl_event;

#define CL_SUCCESS 0
#define CL_FALSE 0
#define CL_TRUE 1
#define CL_DEVICE_TYPE_CPU (1 << 1)
#define CL_DEVICE_TYPE_GPU (1 << 2)
#define CL_DEVICE_TYPE_ACCELERATOR (1 << 3)
#define CL_DEVICE_TYPE_ALL 0xFFFFFFFF
#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)

#ifdef __cplusplus
extern "C" {
#endif
cl_int clFinish(cl_command_queue queue);
cl_int clWaitForEvents(cl_uint num_events, const cl_event* events);
#ifdef __cplusplus
}
#endif
#endif
