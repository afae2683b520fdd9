// The reference's on-disk network format: topo.bin, params.bin, forcings.bin
// in one directory, as written by water-prediction/t-route/wavefront/
// gen_network.py:292-337 and read by wavefront_mc.cu:597-632 (load_topo) and
// :655-672 (params, forcings). All values little-endian.
//
//   topo.bin      int32 n_reaches, n_segments, n_levels, max_upstream;
//                 int32 reach_seg_start[R], reach_seg_len[R], reach_level[R],
//                 reach_n_up[R], reach_up_ptr[R+1], reach_up_idx[nnz],
//                 level_ptr[L+1], level_reach[R]
//   params.bin    float32 [S][8] = dx, bw, tw, twcc, n_ch, ncc, cs, s0
//                 (gen_network.py:319-321 writes float32 although its header
//                 comment says float64; the reader, wavefront_mc.cu:655, reads
//                 float ChParams)
//   forcings.bin  int32 n_ts; float32 qlat[n_ts][S], qup0[R], qdp0[S], dp0[S]
//
// Unlike the reference's reader, a short or inconsistent file is an error
// (TROUTE_EIO / TROUTE_ETOPO) instead of a silent partial read or exit(1).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "troute_internal.h"

namespace {

bool host_little_endian()
{
    const uint32_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

struct File {
    FILE* f = nullptr;
    std::string path;
    ~File()
    {
        if (f) std::fclose(f);
    }
};

int open_file(File& F, const char* dir, const char* name, const char* mode)
{
    F.path = std::string(dir) + "/" + name;
    F.f = std::fopen(F.path.c_str(), mode);
    if (!F.f) return set_error(TROUTE_EIO, "cannot open %s", F.path.c_str());
    return TROUTE_OK;
}

int read_exact(File& F, void* dst, size_t elem, size_t n)
{
    if (n == 0) return TROUTE_OK;
    const size_t got = std::fread(dst, elem, n, F.f);
    if (got != n) return set_error(TROUTE_EIO, "%s: short read (%zu of %zu items)", F.path.c_str(), got, n);
    return TROUTE_OK;
}

int write_exact(File& F, const void* src, size_t elem, size_t n)
{
    if (n == 0) return TROUTE_OK;
    if (!src) return set_error(TROUTE_EINVAL, "%s: null array", F.path.c_str());
    if (std::fwrite(src, elem, n, F.f) != n) return set_error(TROUTE_EIO, "%s: write failed", F.path.c_str());
    return TROUTE_OK;
}

int at_end(File& F)
{
    const int c = std::fgetc(F.f);
    if (c != EOF) return set_error(TROUTE_EIO, "%s: trailing bytes after the expected content", F.path.c_str());
    return TROUTE_OK;
}

template <typename T>
T* alloc_array(size_t n)
{
    return static_cast<T*>(std::calloc(n ? n : 1, sizeof(T)));
}

}  // namespace

extern "C" void troute_free_network(troute_netfile* n)
{
    if (!n) return;
    for (void* p : {(void*)n->reach_seg_start, (void*)n->reach_seg_len, (void*)n->reach_level, (void*)n->reach_n_up,
                    (void*)n->reach_up_ptr, (void*)n->reach_up_idx, (void*)n->level_ptr, (void*)n->level_reach,
                    (void*)n->params, (void*)n->qlat, (void*)n->qup0, (void*)n->qdp0, (void*)n->dp0})
        std::free(p);
    std::free(n);
}

// Structural checks of what was read: CSR monotone and in range, reach_n_up
// and reach_level consistent with it, the level CSR a permutation of the
// reaches in level order, segment ranges inside [0, n_segments).
static int check_netfile(const troute_netfile& n)
{
    const int R = n.n_reaches, S = n.n_segments, L = n.n_levels;
    if (n.reach_up_ptr[0] != 0) return set_error(TROUTE_ETOPO, "topo.bin: reach_up_ptr[0] != 0");
    for (int r = 0; r < R; ++r) {
        const int a = n.reach_up_ptr[r], b = n.reach_up_ptr[r + 1];
        if (b < a) return set_error(TROUTE_ETOPO, "topo.bin: reach_up_ptr decreases at reach %d", r);
        if (n.reach_n_up[r] != b - a) return set_error(TROUTE_ETOPO, "topo.bin: reach_n_up[%d] disagrees with the CSR", r);
        if (n.reach_n_up[r] > n.max_upstream)
            return set_error(TROUTE_ETOPO, "topo.bin: reach %d has more than max_upstream upstream reaches", r);
        if (n.reach_seg_start[r] < 0 || n.reach_seg_len[r] < 0 ||
            (long long)n.reach_seg_start[r] + n.reach_seg_len[r] > (long long)S)
            return set_error(TROUTE_ETOPO, "topo.bin: segments of reach %d outside [0, n_segments)", r);
        if (n.reach_level[r] < 0 || n.reach_level[r] >= L)
            return set_error(TROUTE_ETOPO, "topo.bin: level of reach %d outside [0, n_levels)", r);
        for (int k = a; k < b; ++k) {
            const int u = n.reach_up_idx[k];
            if (u < 0 || u >= R) return set_error(TROUTE_ETOPO, "topo.bin: upstream index %d of reach %d", u, r);
            if (n.reach_level[u] >= n.reach_level[r])
                return set_error(TROUTE_ETOPO, "topo.bin: reach %d is not on a later level than its upstream %d", r, u);
        }
    }
    if (n.level_ptr[0] != 0 || n.level_ptr[L] != R) return set_error(TROUTE_ETOPO, "topo.bin: level_ptr bounds");
    std::vector<char> seen(R, 0);
    for (int l = 0; l < L; ++l) {
        if (n.level_ptr[l + 1] < n.level_ptr[l]) return set_error(TROUTE_ETOPO, "topo.bin: level_ptr decreases");
        for (int i = n.level_ptr[l]; i < n.level_ptr[l + 1]; ++i) {
            const int r = n.level_reach[i];
            if (r < 0 || r >= R || seen[r]) return set_error(TROUTE_ETOPO, "topo.bin: level_reach is not a permutation");
            if (n.reach_level[r] != l) return set_error(TROUTE_ETOPO, "topo.bin: reach %d listed on the wrong level", r);
            seen[r] = 1;
        }
    }
    return TROUTE_OK;
}

extern "C" int troute_read_network(const char* dir, troute_netfile** out)
{
    if (!dir || !out) return set_error(TROUTE_EINVAL, "null argument");
    *out = nullptr;
    if (!host_little_endian()) return set_error(TROUTE_EIO, "the network files are little-endian; this host is not");
    auto* n = static_cast<troute_netfile*>(std::calloc(1, sizeof(troute_netfile)));
    if (!n) return set_error(TROUTE_ENOMEM, "network allocation");
    int rc;
    {
        File F;
        if ((rc = open_file(F, dir, "topo.bin", "rb"))) goto fail;
        int hdr[4];
        if ((rc = read_exact(F, hdr, 4, 4))) goto fail;
        n->n_reaches = hdr[0];
        n->n_segments = hdr[1];
        n->n_levels = hdr[2];
        n->max_upstream = hdr[3];
        if (hdr[0] < 0 || hdr[1] < 0 || hdr[2] < 0 || hdr[3] < 0 || (hdr[0] > 0 && hdr[2] == 0)) {
            rc = set_error(TROUTE_ETOPO, "topo.bin: bad header (%d, %d, %d, %d)", hdr[0], hdr[1], hdr[2], hdr[3]);
            goto fail;
        }
        const size_t R = (size_t)n->n_reaches, L = (size_t)n->n_levels;
        n->reach_seg_start = alloc_array<int>(R);
        n->reach_seg_len = alloc_array<int>(R);
        n->reach_level = alloc_array<int>(R);
        n->reach_n_up = alloc_array<int>(R);
        n->reach_up_ptr = alloc_array<int>(R + 1);
        n->level_ptr = alloc_array<int>(L + 1);
        n->level_reach = alloc_array<int>(R);
        if (!n->reach_seg_start || !n->reach_seg_len || !n->reach_level || !n->reach_n_up || !n->reach_up_ptr ||
            !n->level_ptr || !n->level_reach) {
            rc = set_error(TROUTE_ENOMEM, "topology arrays");
            goto fail;
        }
        if ((rc = read_exact(F, n->reach_seg_start, 4, R)) || (rc = read_exact(F, n->reach_seg_len, 4, R)) ||
            (rc = read_exact(F, n->reach_level, 4, R)) || (rc = read_exact(F, n->reach_n_up, 4, R)) ||
            (rc = read_exact(F, n->reach_up_ptr, 4, R + 1)))
            goto fail;
        const int nnz = n->reach_up_ptr[R];
        if (nnz < 0 || (size_t)nnz > R * (size_t)(n->max_upstream > 0 ? n->max_upstream : 1)) {
            rc = set_error(TROUTE_ETOPO, "topo.bin: %d upstream links for %zu reaches", nnz, R);
            goto fail;
        }
        n->reach_up_idx = alloc_array<int>((size_t)nnz);
        if (!n->reach_up_idx) {
            rc = set_error(TROUTE_ENOMEM, "topology arrays");
            goto fail;
        }
        if ((rc = read_exact(F, n->reach_up_idx, 4, (size_t)nnz)) || (rc = read_exact(F, n->level_ptr, 4, L + 1)) ||
            (rc = read_exact(F, n->level_reach, 4, R)) || (rc = at_end(F)))
            goto fail;
        if ((rc = check_netfile(*n))) goto fail;
    }
    {
        File F;
        if ((rc = open_file(F, dir, "params.bin", "rb"))) goto fail;
        n->params = alloc_array<troute_chparams_f32>((size_t)n->n_segments);
        if (!n->params) {
            rc = set_error(TROUTE_ENOMEM, "parameter array");
            goto fail;
        }
        if ((rc = read_exact(F, n->params, sizeof(troute_chparams_f32), (size_t)n->n_segments)) || (rc = at_end(F)))
            goto fail;
    }
    {
        File F;
        if ((rc = open_file(F, dir, "forcings.bin", "rb"))) goto fail;
        int nts = 0;
        if ((rc = read_exact(F, &nts, 4, 1))) goto fail;
        if (nts < 0) {
            rc = set_error(TROUTE_EIO, "forcings.bin: negative step count");
            goto fail;
        }
        n->n_ts = nts;
        const size_t S = (size_t)n->n_segments, R = (size_t)n->n_reaches;
        n->qlat = alloc_array<float>((size_t)nts * S);
        n->qup0 = alloc_array<float>(R);
        n->qdp0 = alloc_array<float>(S);
        n->dp0 = alloc_array<float>(S);
        if (!n->qlat || !n->qup0 || !n->qdp0 || !n->dp0) {
            rc = set_error(TROUTE_ENOMEM, "forcing arrays");
            goto fail;
        }
        if ((rc = read_exact(F, n->qlat, 4, (size_t)nts * S)) || (rc = read_exact(F, n->qup0, 4, R)) ||
            (rc = read_exact(F, n->qdp0, 4, S)) || (rc = read_exact(F, n->dp0, 4, S)) || (rc = at_end(F)))
            goto fail;
    }
    *out = n;
    return TROUTE_OK;
fail:
    troute_free_network(n);
    return rc;
}

extern "C" int troute_write_network(const char* dir, const troute_netfile* n)
{
    if (!dir || !n) return set_error(TROUTE_EINVAL, "null argument");
    if (!host_little_endian()) return set_error(TROUTE_EIO, "the network files are little-endian; this host is not");
    if (n->n_reaches < 0 || n->n_segments < 0 || n->n_levels < 0 || n->n_ts < 0)
        return set_error(TROUTE_EINVAL, "negative size");
    if (!n->reach_up_ptr || !n->level_ptr) return set_error(TROUTE_EINVAL, "null CSR pointer");
    int rc = check_netfile(*n);
    if (rc) return rc;
    const size_t R = (size_t)n->n_reaches, S = (size_t)n->n_segments, L = (size_t)n->n_levels;
    const size_t nnz = (size_t)n->reach_up_ptr[R];
    {
        File F;
        if ((rc = open_file(F, dir, "topo.bin", "wb"))) return rc;
        const int hdr[4] = {n->n_reaches, n->n_segments, n->n_levels, n->max_upstream};
        if ((rc = write_exact(F, hdr, 4, 4)) || (rc = write_exact(F, n->reach_seg_start, 4, R)) ||
            (rc = write_exact(F, n->reach_seg_len, 4, R)) || (rc = write_exact(F, n->reach_level, 4, R)) ||
            (rc = write_exact(F, n->reach_n_up, 4, R)) || (rc = write_exact(F, n->reach_up_ptr, 4, R + 1)) ||
            (rc = write_exact(F, n->reach_up_idx, 4, nnz)) || (rc = write_exact(F, n->level_ptr, 4, L + 1)) ||
            (rc = write_exact(F, n->level_reach, 4, R)))
            return rc;
    }
    {
        File F;
        if ((rc = open_file(F, dir, "params.bin", "wb"))) return rc;
        if ((rc = write_exact(F, n->params, sizeof(troute_chparams_f32), S))) return rc;
    }
    // without initial state and inflow (the GeoPackage ingest's output) only
    // the topology and the parameters are written
    if (!n->qlat && !n->qup0 && !n->qdp0 && !n->dp0) {
        if (n->n_ts != 0) return set_error(TROUTE_EINVAL, "n_ts > 0 without lateral inflow");
        return TROUTE_OK;
    }
    {
        File F;
        if ((rc = open_file(F, dir, "forcings.bin", "wb"))) return rc;
        const int nts = n->n_ts;
        if ((rc = write_exact(F, &nts, 4, 1)) || (rc = write_exact(F, n->qlat, 4, (size_t)nts * S)) ||
            (rc = write_exact(F, n->qup0, 4, R)) || (rc = write_exact(F, n->qdp0, 4, S)) ||
            (rc = write_exact(F, n->dp0, 4, S)))
            return rc;
    }
    return TROUTE_OK;
}
