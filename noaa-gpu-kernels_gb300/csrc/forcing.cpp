// Lateral-inflow pre-processor: pivots a directory of per-nexus CSV outputs
// (nex-<id>_output.csv, one "step, time, value" row per time step) into the
// [n_ts][n_reaches] float matrix of forcings.bin, in parallel over files.
// Same job and the same parsing rules as the reference's
// water-prediction/t-route/wavefront/data_parsers/parse_qlat_fast_cpp.cpp
// (strip_prefix :41-57, parse_line :59-74, worker loop :147-186):
//  - a file's id is the integer between the first '-' and the next '_' (or '.');
//  - files whose id is not in the reach-id table are counted as missing;
//  - every line of 5 or more characters with a comma gives step = atoi(line)
//    and value = atof(text after the last comma); rows with a step outside
//    [0, n_ts) are ignored, later rows of a file overwrite earlier ones (so a
//    header line, read as step 0, is overwritten by the real step-0 row).
// The directory is listed once (ids looked up there); the files are handed to
// threads in directory order in contiguous chunks. Each file's cells belong
// to one reach, so the result does not depend on the thread count (unless two
// files name the same id, e.g. nex-12 and nex-012: then, as in the reference
// tool, the one written last wins).
#include <dirent.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "troute_internal.h"

namespace {

long long file_id(const std::string& name)
{
    const size_t dash = name.find('-');
    if (dash == std::string::npos) return -1;
    size_t end = name.find('_', dash + 1);
    if (end == std::string::npos) {
        end = name.find('.', dash + 1);
        if (end == std::string::npos) return -1;
    }
    const std::string digits = name.substr(dash + 1, end - dash - 1);
    if (digits.empty()) return -1;
    char* stop = nullptr;
    errno = 0;
    const long v = std::strtol(digits.c_str(), &stop, 10);
    if (stop == digits.c_str() || errno == ERANGE || v < -2147483647L - 1 || v > 2147483647L) return -1;
    return v < 0 ? -1 : v;
}

// One row: step before the first comma, value after the last comma.
bool parse_row(const char* line, size_t len, int* step, float* value)
{
    size_t i = 0;
    while (i < len && line[i] != ',') ++i;
    if (i == len) return false;
    size_t j = len;
    while (j > 0 && line[j - 1] != ',') --j;
    if (j == 0 || j >= len) return false;
    // atoi / atof stop at the first character that does not belong to the number
    *step = std::atoi(line);
    *value = (float)std::atof(line + j);
    return true;
}

}  // namespace

extern "C" int troute_qlat_from_csv(const char* csv_dir, const int64_t* reach_ids, int n_reaches, int n_ts,
                                    int n_threads, float* qlat, long long* matched, long long* missing)
{
    if (!csv_dir || !qlat || (n_reaches > 0 && !reach_ids)) return set_error(TROUTE_EINVAL, "null argument");
    if (n_reaches < 0 || n_ts < 0) return set_error(TROUTE_EINVAL, "negative size");
    std::memset(qlat, 0, (size_t)n_ts * (size_t)n_reaches * sizeof(float));
    std::unordered_map<int64_t, int> index;
    index.reserve((size_t)n_reaches * 2);
    for (int i = 0; i < n_reaches; ++i) index[reach_ids[i]] = i;  // a repeated id maps to its last reach
    // one pass over the directory: the output files and their reaches (the id
    // lookup is done here, once, so the workers only open, read and parse)
    struct CsvFile {
        std::string name;
        int reach;
    };
    std::vector<CsvFile> files;
    long long n_unknown = 0;
    DIR* dir = opendir(csv_dir);
    if (!dir) return set_error(TROUTE_EIO, "cannot list %s: %s", csv_dir, std::strerror(errno));
    const int dfd = dirfd(dir);
    errno = 0;
    for (const dirent* e; (e = readdir(dir)) != nullptr; errno = 0) {
        const char* nm = e->d_name;
        if (std::strncmp(nm, "nex-", 4) != 0 || !std::strstr(nm, "_output.csv")) continue;
        bool regular = e->d_type == DT_REG;
        if (e->d_type == DT_UNKNOWN || e->d_type == DT_LNK) {
            struct stat st;
            regular = fstatat(dfd, nm, &st, 0) == 0 && S_ISREG(st.st_mode);
        }
        if (!regular) continue;
        const long long id = file_id(nm);
        const auto hit = id < 0 ? index.end() : index.find((int64_t)id);
        if (hit == index.end()) {
            ++n_unknown;
            continue;
        }
        files.push_back({nm, hit->second});
    }
    if (errno != 0) {
        const int err = errno;
        closedir(dir);
        return set_error(TROUTE_EIO, "cannot list %s: %s", csv_dir, std::strerror(err));
    }
    if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<long long> n_match{0}, n_miss{n_unknown};
    std::atomic<int> io_error{0};
    const size_t per = (files.size() + (size_t)n_threads - 1) / (size_t)n_threads;
    auto work = [&](size_t b, size_t e) {
        std::vector<char> buf(8192);
        for (size_t fi = b; fi < e; ++fi) {
            const int fd = openat(dfd, files[fi].name.c_str(), O_RDONLY | O_CLOEXEC);
            if (fd < 0) {
                n_miss.fetch_add(1);
                continue;
            }
            size_t got = 0;
            bool failed = false;
            while (true) {
                if (buf.size() < got + 4097) buf.resize(std::max(buf.size() * 2, got + 4097));
                const ssize_t k = read(fd, buf.data() + got, buf.size() - 1 - got);
                if (k < 0) {
                    if (errno == EINTR) continue;
                    failed = true;
                    break;
                }
                if (k == 0) break;
                got += (size_t)k;
            }
            close(fd);
            if (failed) io_error.store(1);
            buf[got] = 0;
            const int reach = files[fi].reach;
            size_t i = 0;
            while (i < got) {
                const size_t ls = i;
                while (i < got && buf[i] != '\n') ++i;
                const size_t len = i - ls;
                if (i < got) ++i;
                if (len < 5) continue;
                int step;
                float v;
                if (!parse_row(buf.data() + ls, len, &step, &v)) continue;
                if (step >= 0 && step < n_ts) qlat[(size_t)step * (size_t)n_reaches + reach] = v;
            }
            n_match.fetch_add(1);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < n_threads; ++t) {
        const size_t b = (size_t)t * per, e = std::min(b + per, files.size());
        if (b >= e) break;
        pool.emplace_back(work, b, e);
    }
    for (auto& th : pool) th.join();
    closedir(dir);
    if (matched) *matched = n_match.load();
    if (missing) *missing = n_miss.load();
    if (io_error.load()) return set_error(TROUTE_EIO, "read error in %s", csv_dir);
    return TROUTE_OK;
}

extern "C" int troute_write_forcings(const char* path, int n_ts, int n_reaches, int n_segments, const float* qlat,
                                     const float* qup0, const float* qdp0, const float* dp0)
{
    if (!path || n_ts < 0 || n_reaches < 0 || n_segments < 0) return set_error(TROUTE_EINVAL, "bad arguments");
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_error(TROUTE_EIO, "cannot open %s", path);
    const int32_t nt = n_ts;
    bool ok = std::fwrite(&nt, 4, 1, f) == 1;
    auto put = [&](const float* a, size_t n) {
        if (!ok || n == 0) return;
        if (!a) {
            ok = false;
            return;
        }
        ok = std::fwrite(a, 4, n, f) == n;
    };
    put(qlat, (size_t)n_ts * (size_t)n_segments);
    put(qup0, (size_t)n_reaches);
    put(qdp0, (size_t)n_segments);
    put(dp0, (size_t)n_segments);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return set_error(TROUTE_EIO, "writing %s failed (or a null array)", path);
    return TROUTE_OK;
}
