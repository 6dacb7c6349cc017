#include "eager.cuh"
#include "stream.cuh"
namespace sjbg {
}
using namespace sjbg;
extern "C" {
int sjbg_stream_open(sjbg_handle *h, uint64_t) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
int sjbg_stream_push(sjbg_handle *h, const sjbg_tuple *, uint64_t, int, uint32_t) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
int sjbg_stream_poll(sjbg_handle *h, sjbg_window_result *, uint32_t, uint32_t *) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
int sjbg_stream_close(sjbg_handle *h, sjbg_stream_stats *) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
}
