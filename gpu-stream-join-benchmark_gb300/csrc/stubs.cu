#include "eager.cuh"
#include "stream.cuh"
namespace sjbg {
int eager_init(sjbg_handle *h) { return fail(h, SJBG_E_UNSUPPORTED, "eager not built yet"); }
}
using namespace sjbg;
extern "C" {
int sjbg_eager_execute(sjbg_handle *h, const sjbg_tuple *, uint64_t, int, uint32_t, uint64_t *) { return fail(h, SJBG_E_UNSUPPORTED, "eager not built yet"); }
int sjbg_eager_clear_states(sjbg_handle *h) { return fail(h, SJBG_E_UNSUPPORTED, "eager not built yet"); }
int sjbg_eager_window_result(sjbg_handle *h, sjbg_pair *, uint64_t, sjbg_window_result *) { return fail(h, SJBG_E_UNSUPPORTED, "eager not built yet"); }
int sjbg_eager_end_of_stream(sjbg_handle *h) { return fail(h, SJBG_E_UNSUPPORTED, "eager not built yet"); }
int sjbg_eager_run(sjbg_handle *h, const sjbg_tuple *, const sjbg_tuple *, uint64_t, uint32_t, uint64_t *, sjbg_window_result *, uint32_t) { return fail(h, SJBG_E_UNSUPPORTED, "eager not built yet"); }
int sjbg_stream_open(sjbg_handle *h, uint64_t) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
int sjbg_stream_push(sjbg_handle *h, const sjbg_tuple *, uint64_t, int, uint32_t) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
int sjbg_stream_poll(sjbg_handle *h, sjbg_window_result *, uint32_t, uint32_t *) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
int sjbg_stream_close(sjbg_handle *h, sjbg_stream_stats *) { return fail(h, SJBG_E_UNSUPPORTED, "stream not built yet"); }
}
