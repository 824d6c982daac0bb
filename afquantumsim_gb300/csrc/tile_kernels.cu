// Shared-memory tile passes (gate runs staged on chip).  Until the tile
// engine is in place the planner issues one pass per gate.
#include "aqsg_internal.h"

namespace aqsg {

int tile_max_bits(int dtype) { return dtype == AQSG_C64 ? 14 : 13; }

int run_tiled(aqsg_state_s* st, const std::vector<LOp>& ops) {
    for (const LOp& o : ops)
        if (int rc = launch_lop(st, o)) return rc;
    return AQSG_OK;
}

}  // namespace aqsg
