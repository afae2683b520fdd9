// Compiles the reference's own reach-parallel CPU routine, unmodified, as a
// host-only library so the oracle can be checked against it bit-for-bit.
// TEST INFRASTRUCTURE ONLY (see troute_oracle.h). REF_ROOT is the reference
// checkout; the file is included from there, never copied.
#define main troute_reference_main_unused
#include REF_MC_FILE
#undef main

extern "C" void ref_cpu_mc(const void* p, const double* ql, const int* rs, const int* rl,
                           const double* qu, const double* qd, const double* dp,
                           double* qo, double* vo, double* dpo,
                           double uq, double dt, int nr)
{
    // cpu_mc: water-prediction/t-route/troute_mc_final.cu:167-252
    cpu_mc(static_cast<const ChParams*>(p), ql, rs, rl, qu, qd, dp, qo, vo, dpo, uq, dt, nr);
}
