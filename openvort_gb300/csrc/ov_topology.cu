// ov_topology.cu - topology passes (reconnect, remesh, small loops, smoothing).
#include "ov_internal.cuh"

extern "C" {
int ov_eliminate_small_loops(ov_ctx *c) { return ov_fail(c, OV_ERR_STATE, "not built yet"); }
int ov_reconnect(ov_ctx *c, double, int *, int *, int *, int) { return ov_fail(c, OV_ERR_STATE, "not built yet"); }
int ov_remesh(ov_ctx *c, double, double, double) { return ov_fail(c, OV_ERR_STATE, "not built yet"); }
int ov_smooth(ov_ctx *c) { return ov_fail(c, OV_ERR_STATE, "not built yet"); }
int ov_step(ov_ctx *c, double, double) { return ov_fail(c, OV_ERR_STATE, "not built yet"); }
}
