/* Minimal type-only stand-in for the OpenCL header so that the reference's
 * CPU-only sources (generator, validators, DP planner) compile for the oracle
 * pin.  No OpenCL entry point is declared: the pinned sources call none. */
#ifndef QG_REF_STUB_OPENCL_H
#define QG_REF_STUB_OPENCL_H
#include <stdint.h>
#include <stddef.h>
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint64_t cl_ulong;
typedef uint64_t cl_bitfield;
typedef cl_bitfield cl_mem_flags;
typedef cl_bitfield cl_device_type;
typedef struct _qg_stub_mem *cl_mem;
typedef struct _qg_stub_event *cl_event;
typedef struct _qg_stub_kernel *cl_kernel;
typedef struct _qg_stub_context *cl_context;
typedef struct _qg_stub_program *cl_program;
typedef struct _qg_stub_queue *cl_command_queue;
typedef struct _qg_stub_platform *cl_platform_id;
typedef struct _qg_stub_device *cl_device_id;
#define CL_SUCCESS 0
#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)
#endif
