// gen.cu - synthetic stream generation in device memory (same draws as the
// host generator in sjbg_gen.h, so device-made inputs equal host-made ones).
#include "runtime.h"

namespace sjbg {

__global__ void gen_kernel(sjbg_tuple *out, uint64_t first, uint64_t n, uint64_t seed, uint64_t domain,
                           const uint64_t *table, uint64_t perm_seed) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t g = first + i;
        uint32_t key;
        if (table) key = sjbg_perm(sjbg_zipf_rank(table, domain, sjbg_rand64(seed, g)), domain, perm_seed);
        else key = sjbg_uniform_key(seed, g, domain);
        uint4 v;
        v.x = key;
        v.y = (uint32_t)g;
        v.z = (uint32_t)g;
        v.w = (uint32_t)(g >> 32);
        reinterpret_cast<uint4 *>(out)[i] = v;
    }
}

int generate_device(sjbg_handle *h, sjbg_tuple *out, uint64_t first, uint64_t n, uint64_t seed, uint64_t domain,
                    const uint64_t *table, uint64_t perm_seed) {
    if (n == 0) return SJBG_OK;
    const uint32_t blocks = (uint32_t)std::min<uint64_t>((n + 255) / 256, (uint64_t)h->num_sms * 16);
    SJBG_CK(h, launch(h, "generate", gen_kernel, dim3(blocks), dim3(256), 0, out, first, n, seed, domain, table,
                      perm_seed));
    return SJBG_OK;
}

}  // namespace sjbg
