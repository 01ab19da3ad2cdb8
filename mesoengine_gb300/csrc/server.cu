// server.cu -- placeholder; replaced by the serving loop.
#include "meso_internal.h"
using namespace meso;
extern "C" {
meso_status meso_server_create(meso_ctx*, const meso_server_config*, meso_scene* const*, uint32_t, meso_server**) { return fail(MESO_ERR_NOT_READY, "server not built"); }
meso_status meso_server_submit(meso_server*, const meso_request*, uint64_t*) { return fail(MESO_ERR_NOT_READY, "server not built"); }
meso_status meso_server_poll(meso_server*, meso_completion*, uint32_t, uint32_t*) { return fail(MESO_ERR_NOT_READY, "server not built"); }
meso_status meso_server_fetch_hits(meso_server*, uint64_t, meso_hit*, uint64_t) { return fail(MESO_ERR_NOT_READY, "server not built"); }
meso_status meso_server_drain(meso_server*, double) { return fail(MESO_ERR_NOT_READY, "server not built"); }
double meso_server_now(const meso_server*) { return 0.0; }
meso_status meso_server_destroy(meso_server*) { return MESO_OK; }
meso_status meso_autotune(meso_ctx*, const char*) { return fail(MESO_ERR_NOT_READY, "autotune not built"); }
}
