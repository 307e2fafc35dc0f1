// tsk_treeseq_general_stat with the reference's C summary-function callback
// (c/tskit/trees.h:1032-1036, c/tskit/trees.c:2035-2095), over the device
// sweeps: the sweep lists the states it meets, the callback is called on the
// host once per listed state, and the values are integrated on the device.
//
// Weights that are all 0 or 1 (each column a set of samples) take the
// counting sweep, which lists each distinct count vector once; other weights
// (and node mode) take the weighted sweep, which lists every state an item, a
// site allele or a leaf needs.  For branch and node mode without
// TSG_STAT_POLARISED the value at a state x is f(x) + f(total - x), as the
// reference's unpolarised wrapper computes it (c/tskit/trees.c:1944-1972).

#include <vector>

#include "tsg_internal.cuh"

namespace {

// f at every listed state (num_states x K doubles), into F (num_states x M)
int call_summary(tsg_general_stat_func_t *f, void *params, uint64_t K, uint64_t M,
    const std::vector<double> &states, int64_t U, bool complement,
    const std::vector<double> &total, std::vector<double> &F)
{
    std::vector<double> y((size_t) M), xc((size_t) K);
    F.assign((size_t) (U * (int64_t) M), 0.0);
    for (int64_t i = 0; i < U; i++) {
        const double *x = states.data() + i * (int64_t) K;
        double *out = F.data() + i * (int64_t) M;
        int ret = f(K, x, M, out, params);
        if (ret != 0) {
            return ret;
        }
        if (complement) {
            for (uint64_t k = 0; k < K; k++) {
                xc[k] = total[k] - x[k];
            }
            ret = f(K, xc.data(), M, y.data(), params);
            if (ret != 0) {
                return ret;
            }
            for (uint64_t m = 0; m < M; m++) {
                out[m] += y[m];
            }
        }
    }
    return 0;
}

}  // namespace

extern "C" {

int tsg_treeseq_general_stat(const tsg_treeseq_t *self, uint64_t state_dim,
    const double *sample_weights, uint64_t result_dim, tsg_general_stat_func_t *f,
    void *f_params, uint64_t num_windows, const double *windows, uint32_t options,
    double *result)
{
    bool site = (options & TSG_STAT_SITE) != 0;
    const bool branch = (options & TSG_STAT_BRANCH) != 0;
    const bool node = (options & TSG_STAT_NODE) != 0;
    if (!(site || branch || node)) {
        site = true;  // the reference's default mode
        options |= TSG_STAT_SITE;
    }
    if ((int) site + (int) branch + (int) node > 1 || (options & TSG_STAT_BOTH_MODES)) {
        return TSG_ERR_MULTIPLE_STAT_MODES;
    }
    if (state_dim < 1) {
        return TSG_ERR_BAD_STATE_DIMS;
    }
    if (result_dim < 1) {
        return TSG_ERR_BAD_RESULT_DIMS;
    }
    if (f == nullptr || sample_weights == nullptr || result == nullptr) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    if (state_dim > TSG_MAX_SAMPLE_SETS) {
        return TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    double default_windows[2] = {0.0, self->v.sequence_length};
    if (windows == nullptr) {
        num_windows = 1;
        windows = default_windows;
    }
    const uint64_t K = state_dim, M = result_dim;
    const int64_t n = self->v.num_samples;
    std::vector<double> total((size_t) K, 0.0);
    bool zero_one = !node;
    std::vector<int64_t> column_count((size_t) K, 0);
    for (int64_t j = 0; j < n; j++) {
        for (uint64_t k = 0; k < K; k++) {
            const double w = sample_weights[j * (int64_t) K + (int64_t) k];
            total[k] += w;
            if (w == 1.0) {
                column_count[k]++;
            } else if (w != 0.0) {
                zero_one = false;
            }
        }
    }
    for (uint64_t k = 0; k < K && zero_one; k++) {
        zero_one = column_count[k] > 0;
    }
    const bool complement = (branch || node) && !(options & TSG_STAT_POLARISED);

    tsg_general_t *g = nullptr;
    int64_t U = 0;
    std::vector<double> states;
    int ret = 0;
    if (zero_one) {
        // each column a sample set: the sample nodes in sample order
        std::vector<int32_t> sample_node((size_t) n, -1);
        for (size_t u = 0; u < self->h_sample_index.size(); u++) {
            const int32_t s = self->h_sample_index[u];
            if (s >= 0 && s < n) {
                sample_node[(size_t) s] = (int32_t) u;
            }
        }
        std::vector<uint64_t> sizes((size_t) K);
        std::vector<int32_t> sets;
        for (uint64_t k = 0; k < K; k++) {
            sizes[k] = (uint64_t) column_count[k];
            for (int64_t j = 0; j < n; j++) {
                if (sample_weights[j * (int64_t) K + (int64_t) k] == 1.0) {
                    sets.push_back(sample_node[(size_t) j]);
                }
            }
        }
        ret = tsg_general_stat_prepare(&g, self, K, sizes.data(), sets.data(), M, num_windows,
            windows, options, &U);
        if (ret == TSG_ERR_TOO_MANY_SAMPLE_SETS) {
            zero_one = false;  // counts beyond the counting sweep: weighted sweep
        } else if (ret != 0) {
            return ret;
        } else {
            std::vector<int32_t> counts((size_t) (U * (int64_t) K));
            ret = tsg_general_stat_states(g, counts.data());
            states.assign(counts.begin(), counts.end());
        }
    }
    if (!zero_one) {
        ret = tsg_general_weighted_prepare(&g, self, K, sample_weights, M, num_windows, windows,
            options, &U);
        if (ret != 0) {
            return ret;
        }
        states.assign((size_t) (U * (int64_t) K), 0.0);
        ret = tsg_general_weighted_states(g, states.data());
    }
    std::vector<double> F;
    if (ret == 0) {
        ret = call_summary(f, f_params, K, M, states, U, complement, total, F);
    }
    if (ret == 0) {
        ret = tsg_general_stat_finish(g, F.data(), result);
    }
    tsg_general_stat_free(g);
    return ret;
}

}  // extern "C"
