// Placeholder until the reference solver kernels land.
#include "reference.h"
namespace mhdproj {
struct RefState {};
int ref_create(RefState**, const mhdproj_grid*, const mhdproj_options*, cudaStream_t, std::string& err) {
    err = "reference solver not available in this build";
    return MHDPROJ_ERR_INVALID;
}
void ref_destroy(RefState*) {}
void ref_set_stream(RefState*, cudaStream_t) {}
int ref_set_topology(RefState*, const uint32_t*, uint32_t, std::string&) { return MHDPROJ_ERR_INVALID; }
int ref_set_coefficients(RefState*, const float*, float, float, std::string&) { return MHDPROJ_ERR_INVALID; }
int ref_set_phase_drag(RefState*, const float*, float, float, std::string&) { return MHDPROJ_ERR_INVALID; }
int ref_project(RefState*, const float*, const float*, const float*, float*, float*, float*, float*, float, int,
                mhdproj_stats*, std::string&) { return MHDPROJ_ERR_INVALID; }
int ref_apply_operator(RefState*, const float*, float*, std::string&) { return MHDPROJ_ERR_INVALID; }
int ref_apply_preconditioner(RefState*, const float*, float*, std::string&) { return MHDPROJ_ERR_INVALID; }
int ref_copy_coefficients(RefState*, float*, std::string&) { return MHDPROJ_ERR_INVALID; }
int ref_copy_potential(RefState*, double*, std::string&) { return MHDPROJ_ERR_INVALID; }
}  // namespace mhdproj
