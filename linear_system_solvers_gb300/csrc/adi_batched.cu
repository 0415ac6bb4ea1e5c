// adi_batched.cu -- batched persistent-kernel solver (lss_adi_batch_*).
#include "adi_batched.hpp"

using namespace lss_gb300;

struct lss_adi_batch {};

extern "C" {
int lss_adi_batch_create(const lss_adi_problem *, int, lss_adi_batch **b)
{
    if (b) *b = nullptr;
    return set_error(LSS_ADI_EUNSUPPORTED, "batch: not built yet");
}
int lss_adi_batch_run(lss_adi_batch *, int, void *) { return set_error(LSS_ADI_EUNSUPPORTED, "batch: not built yet"); }
int lss_adi_batch_graph_launch(lss_adi_batch *, int, void *) { return set_error(LSS_ADI_EUNSUPPORTED, "batch: not built yet"); }
int lss_adi_batch_run_host(lss_adi_batch *, int, const void *, double *, double *, void *)
{
    return set_error(LSS_ADI_EUNSUPPORTED, "batch: not built yet");
}
int lss_adi_batch_results(lss_adi_batch *, double *, double *, int *) { return set_error(LSS_ADI_EUNSUPPORTED, "batch: not built yet"); }
int lss_adi_batch_surface(lss_adi_batch *, int, void *) { return set_error(LSS_ADI_EUNSUPPORTED, "batch: not built yet"); }
int lss_adi_batch_launch_count(const lss_adi_batch *) { return 0; }
void lss_adi_batch_destroy(lss_adi_batch *b) { delete b; }
}
