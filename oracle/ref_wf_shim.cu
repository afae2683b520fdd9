// Compiles the reference's own FP64 tree-routing CPU routine, unmodified, as a
// host-only library (see ref_mc_shim.cu). TEST INFRASTRUCTURE ONLY.
#define main troute_reference_main_unused
#include REF_WF_FILE
#undef main

extern "C" void ref_cpu_wavefront_fp64(
    const void* params, const int* reach_seg_start, const int* reach_seg_len,
    const int* reach_up_ptr, const int* reach_up_idx, const int* level_ptr,
    const int* level_reach, int n_reaches, int n_levels, int n_segments,
    const float* qlat_ts, const float* qdp0_seg, const float* dp0_seg,
    const float* reach_last0, double* qdc_seg_out_d, double* reach_last_out_d,
    int n_timesteps, double dt)
{
    // cpu_wavefront_fp64: water-prediction/t-route/wavefront/wavefront_mc.cu:495-564
    cpu_wavefront_fp64(static_cast<const ChParams*>(params), reach_seg_start, reach_seg_len,
                       reach_up_ptr, reach_up_idx, level_ptr, level_reach, n_reaches,
                       n_levels, n_segments, qlat_ts, qdp0_seg, dp0_seg, reach_last0,
                       qdc_seg_out_d, reach_last_out_d, n_timesteps, dt);
}
