// Multigrid solver driver (filled in below the cascadic path).
#include "epr_context.h"

namespace epr {

bool solve_multigrid(Context &c)
{
    c.fail(EPR_ERR_STATE, "multigrid solver not available in this build");
    return false;
}

}  // namespace epr
