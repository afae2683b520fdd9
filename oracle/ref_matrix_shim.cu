// Compiles the reference's matrix-form coefficient and matrix-build functions
// (water-prediction/t-route/wavefront/linear_mc_matrix.cu), unmodified, as a
// host-only library (see ref_mc_shim.cu). TEST INFRASTRUCTURE ONLY.
#define main troute_reference_matrix_main_unused
#include REF_MATRIX_FILE
#undef main

extern "C" void ref_matrix_coeffs(const void* params, int n, float dt, float* c1, float* c2, float* c3, float* c4oq)
{
    // compute_mc_coeffs_cpu: linear_mc_matrix.cu:56-86
    const ChParams* p = static_cast<const ChParams*>(params);
    for (int i = 0; i < n; ++i) compute_mc_coeffs_cpu(p[i], dt, c1[i], c2[i], c3[i], c4oq[i]);
}

// build_propagation_matrices (linear_mc_matrix.cu:129-216); the matrices are
// kept here until ref_matrix_fetch copies them out.
static Matrix g_ref_PQ, g_ref_Pq;

extern "C" void ref_matrix_build(int n_reaches, const int* up_ptr, const int* up_idx, const float* c1,
                                 const float* c2, const float* c3, const float* c4oq, float tol, int* nnz_Q,
                                 int* nnz_q)
{
    std::vector<int> p(up_ptr, up_ptr + n_reaches + 1), ix(up_idx, up_idx + up_ptr[n_reaches]);
    std::vector<float> a(c1, c1 + n_reaches), b(c2, c2 + n_reaches), c(c3, c3 + n_reaches), d(c4oq, c4oq + n_reaches);
    build_propagation_matrices(n_reaches, p, ix, a, b, c, d, tol, g_ref_PQ, g_ref_Pq);
    *nnz_Q = g_ref_PQ.rowptr.back();
    *nnz_q = g_ref_Pq.rowptr.back();
}

extern "C" void ref_matrix_fetch(int which, int* ptr, int* col, float* val)
{
    const Matrix& m = which ? g_ref_Pq : g_ref_PQ;
    std::copy(m.rowptr.begin(), m.rowptr.end(), ptr);
    std::copy(m.colind.begin(), m.colind.end(), col);
    std::copy(m.values.begin(), m.values.end(), val);
}
