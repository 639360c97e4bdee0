// Receiver-side (adjoint) propagation: RTM imaging and FWI gradients.
#include <cuda_runtime.h>

#include "../../include/pam.h"
#include "pam_engine.h"

extern "C" {

int pam_rtm(pam_engine* e, int, const int*, const int*, const float*, int, int, void*) {
    return e ? e->fail(PAM_E_UNSUPPORTED, "pam_rtm is not available in this build") : PAM_E_ARG;
}
int pam_rtm_result(pam_engine* e, float*, float*, int) {
    return e ? e->fail(PAM_E_UNSUPPORTED, "pam_rtm_result is not available in this build") : PAM_E_ARG;
}
int pam_rtm_reset(pam_engine* e) {
    return e ? e->fail(PAM_E_UNSUPPORTED, "pam_rtm_reset is not available in this build") : PAM_E_ARG;
}
int pam_fwi_gradient(pam_engine* e, int, const int*, const int*, const float*, int, int, double*, void*) {
    return e ? e->fail(PAM_E_UNSUPPORTED, "pam_fwi_gradient is not available in this build") : PAM_E_ARG;
}
int pam_fwi_result(pam_engine* e, float*, float*) {
    return e ? e->fail(PAM_E_UNSUPPORTED, "pam_fwi_result is not available in this build") : PAM_E_ARG;
}
int pam_misfit_gradient(pam_engine* e, int, const int*, const int*, const float*, int, int, double*, float*, void*) {
    return e ? e->fail(PAM_E_UNSUPPORTED, "pam_misfit_gradient is not available in this build") : PAM_E_ARG;
}

}  // extern "C"
