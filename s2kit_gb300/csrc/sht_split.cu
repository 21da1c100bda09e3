// sht_split.cu -- split-precision real-field pipeline (placeholder until the tensor-core path lands)
#include "s2g_internal.h"
namespace s2g {
void free_split(Tables* t) { (void)t; }
size_t split_work_bytes(int bw, int batch) { (void)bw; (void)batch; return 256; }
int fst_split(Tables*, const float*, float*, float*, int, int, void*, cudaStream_t) {
    return fail(S2G_ERR_UNSUPPORTED, "split path not built");
}
int inv_fst_split(Tables*, const float*, const float*, float*, int, int, void*, cudaStream_t) {
    return fail(S2G_ERR_UNSUPPORTED, "split path not built");
}
}  // namespace s2g
