// crg_host.h -- host-side entry points shared between crg_api.cu and crg_server.cu (not part
// of the C ABI).
#pragma once
#include <cstdint>

#include "../../include/crg.h"

namespace crg {

// crg_step split in two so that a caller driving several handles can enqueue all of their
// launches before waiting for any: step_launch issues n_steps steps (at most 256, no cell
// cycle, no profiling) on the handle's stream without waiting; step_wait waits for them,
// reads the device status and accounts the steps exactly as crg_step does.  A handle with
// steps launched must see step_wait before any other call.
int32_t step_launch(crg_ctx *c, int64_t n_steps);
int32_t step_wait(crg_ctx *c, int64_t n_steps);

}  // namespace crg
