/*
 * qg_plan.h -- the dynamic-programming image / kernel-variant planner
 * (host/dynamic_programming.cpp of the reference) in libqg.so.
 */
#ifndef QG_PLAN_H
#define QG_PLAN_H
#include "qg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Primitive operators, the reference's K_KERNEL_INDEX order
 * (host/dynamic_programming.cpp:30-45). */
enum {
    QG_K_SCAN_LARGE_ARRAY = 0,
    QG_K_SCAN_PRE_SUM = 1,
    QG_K_SCAN_BLOCK_ADD = 2,
    QG_K_FILTER_MAP = 3,
    QG_K_FILTER_WRITE = 4,
    QG_K_SORT = 5,
    QG_K_GROUP_LABEL = 6,
    QG_K_GROUP_WRITE = 7,
    QG_K_AGG = 8,
    QG_K_NUM = 9
};

#define QG_PLAN_MAX_OPS 16
#define QG_PLAN_MAX_IMAGES 16

typedef struct {
    int kernel_id; /* QG_K_* */
    int variant;   /* index among that primitive's variants */
} qg_plan_kernel;

/* One image: a run of consecutive operators planned together (an FPGA
 * bitstream in the reference, struct image_info :274-288). */
typedef struct {
    int num_kernels; /* distinct primitives in the image */
    qg_plan_kernel kernels[QG_PLAN_MAX_OPS];
    int luts, regs, rams, dsps;
    float total_unit_cost, exec_time, freq, mem_inc, reconfig_time;
} qg_plan_image;

typedef struct {
    float exec_time; /* modelled total, the reference's printed "total execution time" */
    int image_num;
    qg_plan_image images[QG_PLAN_MAX_IMAGES];
} qg_plan;

/* One row of a cost table: a variant of primitive kernel_id.  Rows must be
 * grouped by kernel_id in increasing order; mem_add / mem_sub of a
 * primitive's first row feed the reconfiguration model. */
typedef struct {
    const char *name;
    int kernel_id;
    int lut, reg, ram, dsp;
    float unit_cost, mem_add, mem_sub;
} qg_plan_variant;

/* dp_for_selection (host/dynamic_programming.cpp:874-996) over `ops`
 * (QG_K_* list), data size in M tuples (truncated to an integer, as dp_test
 * does). */
QG_API qg_status qg_plan_dp(const int *ops, int n_ops, float size_m, qg_plan *out);
/* dp_test (host/dynamic_programming.cpp:1000-1024): sub_index 0 selection,
 * 1 group-by aggregation, 2 filter + group-by aggregation, 3 pre-scan. */
QG_API qg_status qg_plan_pipeline(int sub_index, float size_m, qg_plan *out);
QG_API const char *qg_plan_variant_name(int kernel_id, int variant);
/* Replace the cost table (NULL restores the reference FPGA model).  With
 * fpga_model = 0 the resource -> frequency model is off (freq = 1), which is
 * how a table of measured GPU kernel costs is planned. */
QG_API qg_status qg_plan_set_table(const qg_plan_variant *rows, int n_rows, int fpga_model);
/* The DP of qg_plan_pipeline over the cost table of the context's learned
 * model (qg_steer_attach, include/qg.h); *variant: the operator variant the
 * plan chose.  The process-wide table is not changed. */
QG_API qg_status qg_steer_plan(qg_ctx *ctx, int sub_index, float size_m, qg_plan *out, int *variant);

#ifdef __cplusplus
}
#endif
#endif /* QG_PLAN_H */
