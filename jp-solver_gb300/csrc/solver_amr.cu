// Three-level block AMR solver (reference: src/tgv3d_amr.cu).
#include "jp.h"
#include "solver.h"

namespace jp {

jp_status amr_create(jp_solver*) { return fail(JP_ERR_UNSUPPORTED, "AMR solver not built yet"); }
void amr_destroy(jp_solver*) {}
jp_status amr_init(jp_solver*) { return fail(JP_ERR_UNSUPPORTED, "AMR solver not built yet"); }
jp_status amr_step(jp_solver*, int64_t) { return fail(JP_ERR_UNSUPPORTED, "AMR solver not built yet"); }
jp_status amr_diag(jp_solver*, double*) { return fail(JP_ERR_UNSUPPORTED, "AMR solver not built yet"); }
jp_status amr_population_count(const jp_solver*, int, int64_t*) { return fail(JP_ERR_UNSUPPORTED, "AMR solver not built yet"); }
jp_status amr_get_populations(jp_solver*, int, int, int, void*, int64_t) { return fail(JP_ERR_UNSUPPORTED, "AMR solver not built yet"); }
jp_status amr_set_populations(jp_solver*, int, int, int, const void*, int64_t) { return fail(JP_ERR_UNSUPPORTED, "AMR solver not built yet"); }

}  // namespace jp
