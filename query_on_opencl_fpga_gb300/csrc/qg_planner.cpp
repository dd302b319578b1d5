// qg_planner.cpp -- the dynamic-programming image / kernel-variant planner.
//
// Port of host/dynamic_programming.cpp (Xtra-Computing/Query_on_OpenCL_FPGA):
// for a linear list of primitive operators, choose the cut points that group
// consecutive operators into "images" (one FPGA bitstream each in the
// reference) and, inside each image, one variant per distinct primitive, so
// that the modelled execution time plus reconfiguration cost is minimal.
//   - cost of an image (recursive_time_compute, :329-394): exhaustive search
//     over the variants of its distinct primitives; time =
//     (sum of unit_cost * multiplicity) * data_size / freq, freq from the
//     summed LUT/REG/RAM/DSP use (compute_freq, :306-327);
//   - DP over cut points (dp_for_selection, :874-996) with a reconfiguration
//     cost before every image but the first (:955).
// The arithmetic keeps the reference's types (float accumulators, double
// literals) and evaluation order so the results match its printout bit for
// bit; this file must be built without floating-point contraction.
//
// The kernel table (QG_PLAN_TABLE) is the reference's measured FPGA model
// (:133-185): one row per primitive variant.  The planner also accepts a
// caller-supplied table through qg_plan_set_table, which is how GPU kernel
// variants with measured costs are planned.
#include <math.h>
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "qg.h"
#include "qg_plan.h"

namespace {

struct Variant {
    const char *name;
    int lut, reg, ram, dsp;
    float unit_cost, mem_add, mem_sub;
};

// kernel_primitive[41] of the reference (dynamic_programming.cpp:133-185),
// grouped by primitive in the K_* order (:30-45).
const float SEL_RATE = 0.4f;  // SELECTION_RATE (:47)
const Variant QG_PLAN_TABLE[41] = {
    {"ScanLargeArrays_kernel_1", 11888, 23356, 165, 8, 9.63f, 1.01f, 0.0f},
    {"ScanLargeArrays_kernel_2", 22915, 45564, 330, 16, 3.5f, 1.01f, 0.0f},
    {"ScanLargeArrays_kernel_4", 45093, 90408, 664, 32, 2.46f, 1.01f, 0.0f},
    {"ScanLargeArrays_kernel_8", 89077, 178812, 1320, 64, 0.88f, 1.01f, 0.0f},
    {"ScanLargeArrays_kernel_10", 111131, 223228, 1650, 80, 0.7f, 1.01f, 0.0f},
    {"prefixSum_kernel", 10598, 20726, 137, 8, 0.001f, 0.01f, 0.0f},
    {"blockAddition_kerne_1_1", 7275, 10305, 80, 0, 1.05f, 0.0f, -1.02f},
    {"blockAddition_kerne_1_2", 7010, 10163, 80, 0, 0.53f, 0.0f, -1.02f},
    {"blockAddition_kerne_2_1", 13689, 19462, 160, 0, 0.66f, 0.0f, -1.02f},
    {"blockAddition_kerne_2_4", 13229, 19500, 160, 0, 0.29f, 0.0f, -1.02f},
    {"blockAddition_kerne_1_8", 7395, 10877, 80, 0, 0.14f, 0.0f, -1.02f},
    {"blockAddition_kerne_4_8", 26997, 40064, 320, 0, 0.12f, 0.0f, -1.02f},
    {"blockAddition_kerne_1_16", 8240, 12108, 80, 0, 0.11f, 0.0f, -1.02f},
    {"blockAddition_kerne_8_4", 50333, 74556, 640, 0, 0.11f, 0.0f, -1.02f},
    {"filterImpl_map_kernel_1", 4719, 7995, 38, 0, 1.07f, 1.0f, 0.0f},
    {"filterImpl_map_kernel_2", 8577, 14842, 76, 0, 0.56f, 1.0f, 0.0f},
    {"filterImpl_map_kernel_4", 16293, 28536, 152, 0, 0.41f, 1.0f, 0.0f},
    {"filterImpl_map_kernel_8", 31725, 55924, 304, 0, 0.4f, 1.0f, 0.0f},
    {"filterImpl_write_kernel_1", 9598, 17788, 130, 0, 3.14f, SEL_RATE, -2.0f},
    {"filterImpl_write_kernel_2", 18335, 34428, 260, 0, 2.02f, SEL_RATE, -2.0f},
    {"filterImpl_write_kernel_4", 35809, 67708, 520, 0, 1.01f, SEL_RATE, -2.0f},
    {"filterImpl_write_kernel_8", 70757, 134268, 1040, 0, 0.55f, SEL_RATE, -2.0f},
    {"sort_global_local_kernel_1_1", 20105, 71480, 473, 0, 147.35f, 0.0f, 0.0f},
    {"sort_global_local_kernel_2_1", 30900, 121843, 770, 0, 86.06f, 0.0f, 0.0f},
    {"sort_global_local_kernel_2_2", 38488, 140664, 922, 0, 94.94f, 0.0f, 0.0f},
    {"sort_global_local_kernel_4_2", 53664, 178306, 1226, 0, 62.86f, 0.0f, 0.0f},
    {"sort_global_local_kernel_8_2", 84016, 253590, 1834, 0, 38.05f, 0.0f, 0.0f},
    {"sort_global_local_kernel_10_2", 99192, 291232, 2138, 0, 26.63f, 0.0f, 0.0f},
    {"scanGroupLabel_kernel_1", 6862, 12824, 66, 4, 5.6f, 1.0f, 0.0f},
    {"scanGroupLabel_kernel_2", 12863, 24500, 132, 8, 5.02f, 1.0f, 0.0f},
    {"scanGroupLabel_kernel_4", 24865, 47852, 264, 16, 6.23f, 1.0f, 0.0f},
    {"scanGroupLabel_kernel_8", 48869, 94556, 528, 32, 3.35f, 1.0f, 0.0f},
    {"scanGroupLabel_kernel_16", 96877, 187964, 1056, 64, 1.46f, 1.0f, 0.0f},
    {"groupByImpl_write_kernel_1", 4173, 11921, 59, 4, 6.69f, SEL_RATE, -2.0f},
    {"groupByImpl_write_kernel_2", 7485, 22694, 118, 8, 6.89f, SEL_RATE, -2.0f},
    {"groupByImpl_write_kernel_4", 14109, 44240, 236, 16, 6.65f, SEL_RATE, -2.0f},
    {"groupByImpl_write_kernel_8", 27357, 87332, 472, 32, 5.04f, SEL_RATE, -2.0f},
    {"parallelAggregate_kernel_1", 18018, 33510, 282, 10, 0.96f, SEL_RATE, -1.0f + SEL_RATE},
    {"parallelAggregate_kernel_2", 35175, 65872, 540, 20, 0.54f, SEL_RATE, -1.0f + SEL_RATE},
    {"parallelAggregate_kernel_4", 69489, 130596, 1056, 40, 0.28f, SEL_RATE, -1.0f + SEL_RATE},
    {"parallelAggregate_kernel_6", 103803, 195320, 1572, 60, 0.2f, SEL_RATE, -1.0f + SEL_RATE},
};
// variants per primitive and first row, K_* order (:197-221)
const int QG_PLAN_COUNT[QG_K_NUM] = {5, 1, 8, 4, 4, 6, 5, 4, 4};
const int QG_PLAN_FIRST[QG_K_NUM] = {0, 5, 6, 14, 18, 22, 28, 33, 37};

// The operator lists of dp_test (:223-272).
const int PIPE_SELECTION[5] = {QG_K_FILTER_MAP, QG_K_SCAN_LARGE_ARRAY, QG_K_SCAN_PRE_SUM,
                               QG_K_SCAN_BLOCK_ADD, QG_K_FILTER_WRITE};
const int PIPE_GROUP_AGG[7] = {QG_K_SORT, QG_K_GROUP_LABEL, QG_K_SCAN_LARGE_ARRAY, QG_K_SCAN_PRE_SUM,
                               QG_K_SCAN_BLOCK_ADD, QG_K_GROUP_WRITE, QG_K_AGG};
const int PIPE_FILTER_GROUP_AGG[12] = {QG_K_FILTER_MAP, QG_K_SCAN_LARGE_ARRAY, QG_K_SCAN_PRE_SUM,
                                       QG_K_SCAN_BLOCK_ADD, QG_K_FILTER_WRITE, QG_K_SORT,
                                       QG_K_GROUP_LABEL, QG_K_SCAN_LARGE_ARRAY, QG_K_SCAN_PRE_SUM,
                                       QG_K_SCAN_BLOCK_ADD, QG_K_GROUP_WRITE, QG_K_AGG};

// Active table (reference FPGA model by default).
struct Table {
    std::vector<Variant> rows;
    std::vector<std::string> names;
    int count[QG_K_NUM];
    int first[QG_K_NUM];
    bool fpga;  // resource -> frequency model applies
};
std::mutex g_mu;
Table g_table;
bool g_init = false;

void ensure_table() {
    if (g_init) return;
    g_table.rows.assign(QG_PLAN_TABLE, QG_PLAN_TABLE + 41);
    g_table.names.clear();
    for (const Variant &v : g_table.rows) g_table.names.push_back(v.name);
    for (int k = 0; k < QG_K_NUM; k++) {
        g_table.count[k] = QG_PLAN_COUNT[k];
        g_table.first[k] = QG_PLAN_FIRST[k];
    }
    g_table.fpga = true;
    g_init = true;
}

// compute_freq (:306-327): MHz from the resource use of an image.
float compute_freq(int luts, int regs, int rams, int dsps) {
    const int luts_all = luts + 35437, regs_all = regs + 54855, rams_all = rams + 283, dsps_all = dsps;
    const float luts_rate = ((float)luts_all) / 636928.0;
    const float regs_rate = ((float)regs_all) / 944128.0;
    const float rams_rate = ((float)rams_all) / 2560.0;
    const float dsps_rate = ((float)dsps_all) / 2560.0;
    const float m0 = luts_rate > regs_rate ? luts_rate : regs_rate;
    const float m1 = rams_rate > dsps_rate ? rams_rate : dsps_rate;
    const float m = m0 > m1 ? m0 : m1;
    float freq;
    if ((luts_rate < 0.85) && (regs_rate < 0.85) && (rams_rate < 0.95))
        freq = -85.69 * m * m - 22.02 * m + 278.97;
    else
        freq = 0.01;
    return freq;
}

struct Search {
    const Table *t;
    int data_size;
    const int *prim;   // distinct primitives of the image, first-occurrence order
    const int *mult;   // their multiplicities
    int n;
    int pick[QG_PLAN_MAX_OPS];
    qg_plan_image best;
};

// recursive_time_compute (:329-394): depth-first over the variant of each
// distinct primitive, keeping the first strictly smaller time.
void search(Search &S, int d, int luts, int regs, int rams, int dsps, float unit_cost_base) {
    const int k = S.prim[d];
    const int cnt = S.t->count[k], first = S.t->first[k];
    for (int i = 0; i < cnt; i++) {
        const Variant &v = S.t->rows[first + i];
        float unit_cost = S.mult[d] * v.unit_cost;
        if (k == QG_K_SORT && S.data_size < 16) unit_cost = unit_cost - (128 - S.data_size) * 0.2;
        S.pick[d] = i;
        if (d == S.n - 1) {
            const float freq = S.t->fpga ? compute_freq(luts + v.lut, regs + v.reg, rams + v.ram, dsps + v.dsp)
                                         : 1.0f;
            const float time = ((unit_cost_base + unit_cost) * (float)S.data_size) / freq;
            if (time < S.best.exec_time) {
                S.best.total_unit_cost = unit_cost_base + unit_cost;
                S.best.exec_time = time;
                S.best.freq = freq;
                S.best.num_kernels = S.n;
                for (int j = 0; j < S.n; j++) {
                    S.best.kernels[j].kernel_id = S.prim[j];
                    S.best.kernels[j].variant = S.pick[j];
                }
                S.best.luts = luts + v.lut;
                S.best.regs = regs + v.reg;
                S.best.rams = rams + v.ram;
                S.best.dsps = dsps + v.dsp;
            }
        } else {
            search(S, d + 1, luts + v.lut, regs + v.reg, rams + v.ram, dsps + v.dsp, unit_cost_base + unit_cost);
        }
    }
}

qg_status plan(const Table &t, const int *ops, int n_ops, int data_size, qg_plan *out) {
    if (n_ops < 1 || n_ops > QG_PLAN_MAX_OPS || !ops || !out) return QG_ERR_INVALID;
    for (int i = 0; i < n_ops; i++)
        if (ops[i] < 0 || ops[i] >= QG_K_NUM) return QG_ERR_INVALID;
    std::vector<float> footprint(n_ops + 1, 0.0f), overhead(n_ops + 1, 0.0f);
    footprint[0] = 1.0;
    std::vector<qg_plan> best(n_ops + 1);
    memset(best.data(), 0, sizeof(qg_plan) * best.size());
    best[0].image_num = 0;
    best[0].exec_time = 0;
    for (int i = 1; i <= n_ops; i++) {
        const Variant &head = t.rows[t.first[ops[i - 1]]];
        overhead[i] = footprint[i - 1] + head.mem_add;
        footprint[i] = overhead[i] + head.mem_sub;
        float time_min = 99999999.9;
        int brk = 0;
        qg_plan_image chosen;
        memset(&chosen, 0, sizeof(chosen));
        for (int j = 0; j < i; j++) {
            const float sub = best[j].exec_time;
            int prim[QG_PLAN_MAX_OPS], mult[QG_PLAN_MAX_OPS], u = 0;
            for (int q = j; q < i; q++) {
                int m = -1;
                for (int r = 0; r < u; r++)
                    if (prim[r] == ops[q]) m = r;
                if (m >= 0) mult[m]++;
                else { prim[u] = ops[q]; mult[u] = 1; u++; }
            }
            Search S;
            memset(&S.best, 0, sizeof(S.best));
            S.t = &t;
            S.data_size = data_size;
            S.prim = prim;
            S.mult = mult;
            S.n = u;
            S.best.exec_time = 99999999.0;
            search(S, 0, 0, 0, 0, 0, 0.0);
            const float img = S.best.exec_time;
            float reconfig = 0.0;
            if (j != 0) reconfig = (0.993 * data_size * 4.0 * overhead[j + 1] + 1914.6) / 1000.0;
            if ((sub + img + reconfig) < time_min) {
                S.best.mem_inc = overhead[j + 1];
                S.best.reconfig_time = reconfig;
                brk = j;
                chosen = S.best;
                time_min = sub + img + reconfig;
            }
        }
        best[i].exec_time = time_min;
        const int prev = best[brk].image_num;
        if (prev + 1 > QG_PLAN_MAX_IMAGES) return QG_ERR_UNSUPPORTED;
        best[i].image_num = prev + 1;
        for (int k = 0; k < prev; k++) best[i].images[k] = best[brk].images[k];
        best[i].images[prev] = chosen;
    }
    *out = best[n_ops];
    return QG_OK;
}

qg_status make_table(const qg_plan_variant *rows, int n_rows, int fpga_model, Table *out);

}  // namespace

extern "C" {

QG_API qg_status qg_plan_dp(const int *ops, int n_ops, float size_m, qg_plan *out) {
    std::lock_guard<std::mutex> lock(g_mu);
    ensure_table();
    const int data_size = (int)(size_m * 1.0);  // dp_test (:1000-1002): data_size is an int
    return plan(g_table, ops, n_ops, data_size, out);
}

QG_API qg_status qg_plan_pipeline(int sub_index, float size_m, qg_plan *out) {
    switch (sub_index) {  // dp_test (:1000-1024)
        case 0: return qg_plan_dp(PIPE_SELECTION, 5, size_m, out);
        case 1: return qg_plan_dp(PIPE_GROUP_AGG, 7, size_m, out);
        case 2: return qg_plan_dp(PIPE_FILTER_GROUP_AGG, 12, size_m, out);
        case 3: return qg_plan_dp(PIPE_SELECTION + 1, 3, size_m, out);
    }
    return QG_ERR_INVALID;
}

QG_API const char *qg_plan_variant_name(int kernel_id, int variant) {
    std::lock_guard<std::mutex> lock(g_mu);
    ensure_table();
    if (kernel_id < 0 || kernel_id >= QG_K_NUM || variant < 0 || variant >= g_table.count[kernel_id])
        return "";
    return g_table.names[g_table.first[kernel_id] + variant].c_str();
}

QG_API qg_status qg_plan_set_table(const qg_plan_variant *rows, int n_rows, int fpga_model) {
    std::lock_guard<std::mutex> lock(g_mu);
    ensure_table();
    if (!rows) {  // back to the reference FPGA model
        g_init = false;
        ensure_table();
        return QG_OK;
    }
    Table t;
    const qg_status st = make_table(rows, n_rows, fpga_model, &t);
    if (st != QG_OK) return st;
    g_table = t;
    return QG_OK;
}

}  // extern "C"

// The DP over one of dp_test's pipelines with a caller-built table, leaving
// the process-wide table alone (the learned variant choice plans with it).
qg_status qg_plan_pipeline_rows(const qg_plan_variant *rows, int n_rows, int fpga_model, int sub_index,
                                float size_m, qg_plan *out) {
    Table t;
    const qg_status st = make_table(rows, n_rows, fpga_model, &t);
    if (st != QG_OK) return st;
    const int data_size = (int)(size_m * 1.0);
    switch (sub_index) {
        case 0: return plan(t, PIPE_SELECTION, 5, data_size, out);
        case 1: return plan(t, PIPE_GROUP_AGG, 7, data_size, out);
        case 2: return plan(t, PIPE_FILTER_GROUP_AGG, 12, data_size, out);
        case 3: return plan(t, PIPE_SELECTION + 1, 3, data_size, out);
    }
    return QG_ERR_INVALID;
}

namespace {
qg_status make_table(const qg_plan_variant *rows, int n_rows, int fpga_model, Table *out) {
    if (!rows || n_rows < QG_K_NUM) return QG_ERR_INVALID;
    Table t;
    for (int k = 0; k < QG_K_NUM; k++) t.count[k] = 0;
    int prev = -1;
    for (int i = 0; i < n_rows; i++) {
        const qg_plan_variant &r = rows[i];
        if (r.kernel_id < 0 || r.kernel_id >= QG_K_NUM || r.kernel_id < prev) return QG_ERR_INVALID;
        if (r.kernel_id != prev) t.first[r.kernel_id] = i;
        prev = r.kernel_id;
        t.count[r.kernel_id]++;
        t.rows.push_back(Variant{nullptr, r.lut, r.reg, r.ram, r.dsp, r.unit_cost, r.mem_add, r.mem_sub});
        t.names.push_back(r.name);
    }
    for (int k = 0; k < QG_K_NUM; k++)
        if (t.count[k] == 0) return QG_ERR_INVALID;
    t.fpga = fpga_model != 0;
    *out = t;
    return QG_OK;
}
}  // namespace
