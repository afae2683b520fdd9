// Compiles the reference's own linearised-MC CPU routine and its coefficient
// function, unmodified, as a host-only library (see ref_mc_shim.cu).
// TEST INFRASTRUCTURE ONLY.
#define main troute_reference_linear_main_unused
#include REF_LIN_FILE
#undef main

extern "C" void ref_linear_coeffs(const void* params, int n, float dt, float* c1, float* c2, float* c3, float* c4oq)
{
    // compute_mc_coeffs: water-prediction/t-route/wavefront/linear_mc.cu:57-100 (host instance)
    const ChParams* p = static_cast<const ChParams*>(params);
    for (int i = 0; i < n; ++i) compute_mc_coeffs(p[i], dt, c1[i], c2[i], c3[i], c4oq[i]);
}

extern "C" void ref_cpu_linear_mc(const float* c1, const float* c2, const float* c3, const float* c4oq,
                                  const int* reach_seg_start, const int* reach_seg_len, const int* reach_up_ptr,
                                  const int* reach_up_idx, const int* level_ptr, const int* level_reach,
                                  int n_reaches, int n_levels, int n_segments, const float* qlat_ts,
                                  const float* q0, float* q_final, int n_timesteps)
{
    // cpu_linear_mc: water-prediction/t-route/wavefront/linear_mc.cu:177-232
    cpu_linear_mc(c1, c2, c3, c4oq, reach_seg_start, reach_seg_len, reach_up_ptr, reach_up_idx, level_ptr,
                  level_reach, n_reaches, n_levels, n_segments, qlat_ts, q0, q_final, n_timesteps);
}
