// matfree.cu -- mixed-precision matrix-free SIMP operator (placeholder).
#include "mg_internal.h"

namespace mg {

int matfree_solve(mg_problem *p, const mg_solve_opts &o, mg_solve_report *rep) {
    (void)p; (void)o; (void)rep;
    set_error("mixed-precision path not built");
    return MG_ENOTSUP;
}

void matfree_free(mg_problem *p) { (void)p; }

}  // namespace mg
