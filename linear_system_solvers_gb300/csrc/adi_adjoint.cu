// adi_adjoint.cu -- adjoint (reverse-mode) of the whole ADI solve.
#include "adi_batched.hpp"

namespace lss_gb300 {

struct adjoint_impl {};

adjoint_solver::adjoint_solver() = default;
adjoint_solver::~adjoint_solver() = default;

int adjoint_solver::init(const lss_adi_problem &) { return set_error(LSS_ADI_EUNSUPPORTED, "adjoint: not built yet"); }
int adjoint_solver::run(const void *, double *, double *, void *, int, int, void *)
{
    return set_error(LSS_ADI_EUNSUPPORTED, "adjoint: not built yet");
}

} // namespace lss_gb300
