// Continuous-batching solve server (filled in below).
#include "crs.cuh"

extern "C" {
int cigpu_server_create(int, size_t, int, int, cigpu_server **out) { if (out) *out = nullptr; return CIGPU_ENOTSUP; }
int cigpu_server_submit(cigpu_server *, const cigpu_request *, uint64_t *) { return CIGPU_ENOTSUP; }
int cigpu_server_poll(cigpu_server *, uint64_t, int, cigpu_result *, double *, double *) { return CIGPU_ENOTSUP; }
int cigpu_server_cancel(cigpu_server *, uint64_t) { return CIGPU_ENOTSUP; }
int cigpu_server_stats(cigpu_server *, int64_t *, int64_t *, int64_t *, size_t *) { return CIGPU_ENOTSUP; }
int cigpu_server_destroy(cigpu_server *) { return CIGPU_OK; }
}
