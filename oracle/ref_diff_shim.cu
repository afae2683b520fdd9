// Compiles the reference's own diffusive-wave CPU routine, unmodified, as a
// host-only library (see ref_mc_shim.cu). TEST INFRASTRUCTURE ONLY.
#define main troute_reference_owp_main_unused
#include REF_OWP_FILE
#undef main

extern "C" void ref_cpu_diffusive_tridiag(const void* rp, const float* dx, const float* diffusivity,
                                          const float* celerity, const float* qp_prev, float* qp_out, int nreach)
{
    // cpu_diffusive_tridiag: water-prediction/owp_extended_kernels.cu:35-91 (arrays [nreach][MAX_NODES])
    cpu_diffusive_tridiag(static_cast<const DiffReachParams*>(rp), dx, diffusivity, celerity, qp_prev, qp_out, nreach);
}

extern "C" int ref_diffusive_max_nodes(void) { return MAX_NODES; }
