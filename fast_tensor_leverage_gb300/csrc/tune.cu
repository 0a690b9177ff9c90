// Runtime selection of kernel variants (the autotuner's choices).
//
// Some kernels exist in several compiled variants that compute the same
// results with different launch shapes; which one is fastest depends on the
// GPU and the problem.  The Python autotuner (fast_tensor_leverage_gb300/
// autotune.py) times them and records its choice here through ftl_tune_set;
// the launchers read it with tuned_variant.  Choices are per device (kernel
// performance is a property of the GPU a launch runs on) and per variant
// class of the family.  Unset entries use the family's default.
//
// Families:
//   FTL_TUNE_DRAW: the FP32 draw on DIAG32 trees (16 < R <= 32); variants
//     0, 1, 2 descend 1, 2, 3 samples per warp in lockstep with the query
//     weights in registers (1: 8 warps per block, 768 threads per SM; 2 and
//     3: 4 warps per block, 512 threads per SM); variants 3, 4, 5 keep the
//     weights in shared memory and descend 3, 4, 6 samples per warp (640,
//     512, 384 threads per SM).  Other ranks and precisions have one variant.
#include <mutex>

#include "ftl_common.cuh"

namespace ftl {

namespace {

constexpr int kMaxDevices = 64;
constexpr int kFamilies = 1;
constexpr int kClasses = 2;
std::mutex g_tune_mutex;
int g_tune[kMaxDevices][kFamilies][kClasses];
bool g_tune_init = false;

// Variant class of (family, R, prec) and its variant count and default.
int variant_class(int family, int R, int prec, int *count, int *dflt) {
    (void)family;
    if (storage_prec(prec) == FTL_PREC_FP32 && node_layout(R, 4) == FTL_LAYOUT_DIAG32) {
        *count = 6;
        *dflt = 2;
        return 1;
    }
    *count = 1;
    *dflt = 0;
    return 0;
}

int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
    return dev;
}

}  // namespace

int tuned_variant(int family, int R, int prec) {
    int count = 1, dflt = 0;
    const int cls = variant_class(family, R, prec, &count, &dflt);
    if (family < 0 || family >= kFamilies) return dflt;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    if (!g_tune_init) return dflt;
    const int v = g_tune[current_device()][family][cls];
    return (v >= 0 && v < count) ? v : dflt;
}

}  // namespace ftl

using namespace ftl;

extern "C" int ftl_tune_variants(int family, int R, int prec, int *count, int *default_variant) {
    FTL_CHECK_ARG(family >= 0 && family < kFamilies, "ftl_tune_variants: unknown family %d", family);
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && valid_prec(prec), "ftl_tune_variants: bad R=%d or precision %d", R,
                  prec);
    int c = 1, d = 0;
    variant_class(family, R, prec, &c, &d);
    if (count) *count = c;
    if (default_variant) *default_variant = d;
    return FTL_OK;
}

extern "C" int ftl_tune_set(int family, int R, int prec, int variant) {
    FTL_CHECK_ARG(family >= 0 && family < kFamilies, "ftl_tune_set: unknown family %d", family);
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && valid_prec(prec), "ftl_tune_set: bad R=%d or precision %d", R, prec);
    int count = 1, dflt = 0;
    const int cls = variant_class(family, R, prec, &count, &dflt);
    FTL_CHECK_ARG(variant >= -1 && variant < count, "ftl_tune_set: variant %d outside [-1, %d)", variant, count);
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    if (!g_tune_init) {
        for (auto &d : g_tune)
            for (auto &f : d)
                for (int &v : f) v = -1;
        g_tune_init = true;
    }
    g_tune[current_device()][family][cls] = variant;  // -1: back to the default
    return FTL_OK;
}

extern "C" int ftl_tune_get(int family, int R, int prec, int *variant) {
    FTL_CHECK_ARG(variant != nullptr, "ftl_tune_get: variant is NULL");
    FTL_CHECK_ARG(family >= 0 && family < kFamilies, "ftl_tune_get: unknown family %d", family);
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && valid_prec(prec), "ftl_tune_get: bad R=%d or precision %d", R, prec);
    *variant = tuned_variant(family, R, prec);
    return FTL_OK;
}
