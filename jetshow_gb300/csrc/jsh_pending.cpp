// Entry points whose implementation lands in later commits; each returns an
// error so a caller never mistakes them for working code.
#include "jsh_context.h"
#define JSH_PENDING(name) do { jsh_set_error(name ": not available in this build"); return JSH_ERR_INVALID; } while (0)
extern "C" int jsh_grid_triangulate(const double*, int64_t, int32_t*, int64_t*) { JSH_PENDING("jsh_grid_triangulate"); }
extern "C" int jsh_grid_upload(jsh_ctx*, const double*, int64_t, const float*, int32_t, const int32_t*, int64_t, int32_t*) { JSH_PENDING("jsh_grid_upload"); }
extern "C" int jsh_grid_interpolate(jsh_ctx*, int32_t, int32_t, const double*, int64_t, double, double*) { JSH_PENDING("jsh_grid_interpolate"); }
extern "C" int jsh_server_create(jsh_ctx*, const jsh_server_config*, jsh_server**) { JSH_PENDING("jsh_server_create"); }
extern "C" void jsh_server_destroy(jsh_server*) {}
extern "C" int jsh_server_submit(jsh_server*, const jsh_model_desc*, const jsh_plane_desc*, const double*, int32_t, const jsh_params*, jsh_request_id*) { JSH_PENDING("jsh_server_submit"); }
extern "C" int jsh_server_poll(jsh_server*, jsh_request_id) { JSH_PENDING("jsh_server_poll"); }
extern "C" int jsh_server_wait(jsh_server*, jsh_request_id, int32_t, jsh_image*, jsh_request_stats*) { JSH_PENDING("jsh_server_wait"); }
extern "C" int jsh_server_cancel(jsh_server*, jsh_request_id) { JSH_PENDING("jsh_server_cancel"); }
extern "C" int jsh_autotune(jsh_ctx*, const jsh_model_desc*, const jsh_plane_desc*, const double*, int32_t, const jsh_params*, jsh_tuning*) { JSH_PENDING("jsh_autotune"); }
