// Dataset container standing in for the HDF5 files of the path (nevpt.h5
// written by stage 1 and read by stage 2, src/koopro4QD.F90:305,369-418,
// 473-477 and src/qdnevpt.F:792-853; the QCMaquis result files whose
// label/value datasets src/rdm_utils.F90:69-227 reads), for builds without
// libhdf5.  Datasets keep the HDF5 names ("/spectrum/results/fourptdm/
// labels_num", "amatIP", ...), element type and Fortran-order dimensions.
//
// File layout (little-endian):
//   "NVPTC1\0\0"                                   8 bytes
//   records, each:
//     u32 name length, name bytes
//     u32 type (1 int32, 2 int64, 3 float64), u32 rank
//     u64 dims[rank] (Fortran order, fastest first), u64 payload bytes
//     payload
// Writing a dataset appends a record; on reading, the last record of a name
// wins (replacing a dataset as the reference's writers do).
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/nvpt2.h"

namespace {

const char kMagic[8] = {'N', 'V', 'P', 'T', 'C', '1', 0, 0};

size_t type_size(int t) { return t == 1 ? 4 : (t == 2 || t == 3) ? 8 : 0; }

struct Rec {
    std::string name;
    uint32_t type = 0, rank = 0;
    uint64_t dims[8] = {0};
    uint64_t bytes = 0;
    long offset = 0;  // payload position
};

// Index of the file's records; false if it is not a container.
bool scan(FILE *f, std::vector<Rec> &out) {
    char m[8];
    if (fread(m, 1, 8, f) != 8 || memcmp(m, kMagic, 8) != 0) return false;
    for (;;) {
        uint32_t len;
        if (fread(&len, 4, 1, f) != 1) return true;  // end of file
        if (len > 4096) return false;
        Rec r;
        r.name.resize(len);
        if (len && fread(&r.name[0], 1, len, f) != len) return false;
        if (fread(&r.type, 4, 1, f) != 1 || fread(&r.rank, 4, 1, f) != 1 || r.rank > 8) return false;
        if (r.rank && fread(r.dims, 8, r.rank, f) != r.rank) return false;
        if (fread(&r.bytes, 8, 1, f) != 1) return false;
        r.offset = ftell(f);
        if (fseek(f, (long)r.bytes, SEEK_CUR) != 0) return false;
        out.push_back(r);
    }
}

int find(const char *path, const char *name, Rec &rec) {
    FILE *f = fopen(path, "rb");
    if (!f) return NVPT_EIO;
    std::vector<Rec> v;
    const bool ok = scan(f, v);
    fclose(f);
    if (!ok) return NVPT_EIO;
    for (auto it = v.rbegin(); it != v.rend(); ++it)
        if (it->name == name) {
            rec = *it;
            return NVPT_OK;
        }
    return NVPT_EINVAL;
}

}  // namespace

extern "C" {

int nvpt_h5c_write(const char *path, const char *name, int type, int rank, const int64_t *dims, const void *data,
                   int append) {
    if (!path || !name || type_size(type) == 0 || rank < 0 || rank > 8 || (rank && !dims)) return NVPT_EINVAL;
    uint64_t count = 1;
    for (int i = 0; i < rank; ++i) {
        if (dims[i] < 0) return NVPT_EINVAL;
        count *= (uint64_t)dims[i];
    }
    const uint64_t bytes = count * type_size(type);
    if (bytes && !data) return NVPT_EINVAL;
    FILE *f = nullptr;
    if (append) {
        f = fopen(path, "r+b");
        if (f) {
            std::vector<Rec> v;
            if (!scan(f, v)) {
                fclose(f);
                return NVPT_EIO;
            }
            fseek(f, 0, SEEK_END);
        }
    }
    if (!f) {
        f = fopen(path, "wb");
        if (!f) return NVPT_EIO;
        if (fwrite(kMagic, 1, 8, f) != 8) {
            fclose(f);
            return NVPT_EIO;
        }
    }
    const uint32_t len = (uint32_t)strlen(name), t = (uint32_t)type, r = (uint32_t)rank;
    bool ok = fwrite(&len, 4, 1, f) == 1 && fwrite(name, 1, len, f) == len && fwrite(&t, 4, 1, f) == 1 &&
              fwrite(&r, 4, 1, f) == 1;
    for (int i = 0; ok && i < rank; ++i) {
        const uint64_t d = (uint64_t)dims[i];
        ok = fwrite(&d, 8, 1, f) == 1;
    }
    ok = ok && fwrite(&bytes, 8, 1, f) == 1 && (bytes == 0 || fwrite(data, 1, bytes, f) == bytes);
    ok = (fclose(f) == 0) && ok;
    return ok ? NVPT_OK : NVPT_EIO;
}

int nvpt_h5c_info(const char *path, const char *name, int *type, int *rank, int64_t *dims) {
    if (!path || !name) return NVPT_EINVAL;
    Rec r;
    const int st = find(path, name, r);
    if (st != NVPT_OK) return st;
    if (type) *type = (int)r.type;
    if (rank) *rank = (int)r.rank;
    if (dims)
        for (uint32_t i = 0; i < r.rank; ++i) dims[i] = (int64_t)r.dims[i];
    return NVPT_OK;
}

int nvpt_h5c_read(const char *path, const char *name, void *data, int64_t nbytes) {
    if (!path || !name || nbytes < 0) return NVPT_EINVAL;
    Rec r;
    const int st = find(path, name, r);
    if (st != NVPT_OK) return st;
    if ((uint64_t)nbytes != r.bytes) return NVPT_EINVAL;
    if (r.bytes == 0) return NVPT_OK;
    if (!data) return NVPT_EINVAL;
    FILE *f = fopen(path, "rb");
    if (!f) return NVPT_EIO;
    const bool ok = fseek(f, r.offset, SEEK_SET) == 0 && fread(data, 1, r.bytes, f) == r.bytes;
    fclose(f);
    return ok ? NVPT_OK : NVPT_EIO;
}

// Sorted entries of a directory (what `ls -1` lists), for the distributed reader.
int nvpt_h5c_list_dir(const char *path, char *buf, int64_t len) {
    if (!path) return -1;
    DIR *d = opendir(path);
    if (!d) return -1;
    std::vector<std::string> names;
    while (dirent *e = readdir(d)) {
        const std::string n = e->d_name;
        if (n != "." && n != "..") names.push_back(n);
    }
    closedir(d);
    std::sort(names.begin(), names.end());
    std::string all;
    for (auto &n : names) all += n + "\n";
    if (buf && len > 0) {
        const size_t k = std::min((size_t)(len - 1), all.size());
        memcpy(buf, all.data(), k);
        buf[k] = 0;
    }
    return (int)all.size() + 1;
}

}  // extern "C"

extern "C" const char *nvpt_context_error_set(nvpt_context *ctx, const char *msg);

namespace {
int rdm_fail(nvpt_context *ctx, int code, const std::string &m) {
    nvpt_context_error_set(ctx, m.c_str());
    return code;
}
bool file_exists(const std::string &p) {
    struct stat sb;
    return stat(p.c_str(), &sb) == 0 && S_ISREG(sb.st_mode);
}
}  // namespace

extern "C" {

// src/rdm_utils.F90:69-227 hdf5_read_rdm_from_resfile on a container file.
int nvpt_read_rdm_from_resfile(nvpt_context *ctx, const char *path, int which, int trans, double *rdm, int64_t ld,
                               int64_t nact, int64_t *read_num_elements) {
    if (!ctx || !path || !rdm || (which != 3 && which != 4)) return NVPT_EINVAL;
    if (!file_exists(path)) return rdm_fail(ctx, NVPT_EIO, std::string("Cannot find QCMaquis result file ") + path);
    const std::string root = which == 4 ? "/spectrum/results/fourptdm"
                                        : (trans ? "/spectrum/results/transition_threeptdm" : "/spectrum/results/threeptdm");
    const std::string lname = root + "/labels_num", vname = root + "/mean/value";
    int lt = 0, lr = 0, vt = 0, vr = 0;
    int64_t ldims[8], vdims[8];
    if (nvpt_h5c_info(path, lname.c_str(), &lt, &lr, ldims) != NVPT_OK || lt != 1 || lr != 2)
        return rdm_fail(ctx, NVPT_EINVAL, "Could not open the RDM dataset " + lname + " in " + path);
    const int64_t rank = ldims[0], nentries = ldims[1];
    if (which == 4 && rank != 8) return rdm_fail(ctx, NVPT_EINVAL, "4-RDM should have 8 indices per entry stored");
    if (which == 3 && rank != 6) return rdm_fail(ctx, NVPT_EINVAL, "3-RDM should have 6 indices per entry stored");
    if (nvpt_h5c_info(path, vname.c_str(), &vt, &vr, vdims) != NVPT_OK || vt != 3 || vr != 1)
        return rdm_fail(ctx, NVPT_EINVAL, "Could not open the RDM dataset " + vname + " in " + path);
    if (vdims[0] != nentries)
        return rdm_fail(ctx, NVPT_EINVAL, "Dataset size mismatch between RDM labels and values in " + std::string(path));
    std::vector<int32_t> labels((size_t)(rank * nentries));
    std::vector<double> values((size_t)nentries);
    if (nvpt_h5c_read(path, lname.c_str(), labels.data(), (int64_t)(labels.size() * 4)) != NVPT_OK ||
        nvpt_h5c_read(path, vname.c_str(), values.data(), (int64_t)(values.size() * 8)) != NVPT_OK)
        return rdm_fail(ctx, NVPT_EIO, std::string("read error in ") + path);
    if (read_num_elements) *read_num_elements = nentries;
    return which == 4 ? nvpt_permute_4rdm(ctx, rdm, nact, labels.data(), values.data(), nentries)
                      : nvpt_permute_3rdm(ctx, rdm, ld, nact, labels.data(), values.data(), nentries, trans);
}

// src/rdm_utils.F90:522-614 read_distributed_rdm: every subdirectory of dir
// (sorted) holding result_name is read in turn until total_elements entries
// have been read.
int nvpt_read_distributed_rdm(nvpt_context *ctx, const char *dir, const char *result_name, int which, int trans,
                              double *rdm, int64_t ld, int64_t nact, int64_t total_elements) {
    if (!ctx || !dir || !result_name) return NVPT_EINVAL;
    const int need = nvpt_h5c_list_dir(dir, nullptr, 0);
    if (need < 0) return rdm_fail(ctx, NVPT_EIO, std::string("Cannot find path ") + dir + ".");
    std::string list((size_t)need, '\0');
    nvpt_h5c_list_dir(dir, &list[0], need);
    int64_t acc = 0;
    size_t pos = 0;
    while (pos < list.size() && list[pos]) {
        const size_t e = list.find('\n', pos);
        if (e == std::string::npos) break;
        const std::string file = std::string(dir) + "/" + list.substr(pos, e - pos) + "/" + result_name;
        pos = e + 1;
        if (!file_exists(file)) continue;
        int64_t k = 0;
        const int st = nvpt_read_rdm_from_resfile(ctx, file.c_str(), which, trans, rdm, ld, nact, &k);
        if (st != NVPT_OK) return st;
        acc += k;
        if (acc == total_elements) break;
    }
    if (acc != total_elements)
        return rdm_fail(ctx, NVPT_EINVAL,
                        acc == 0 ? "Did not find any QCMaquis HDF5 result files. Did you specify the correct path?"
                                 : "Mismatch in the number of RDM elements. Could read only " + std::to_string(acc) +
                                       " out of " + std::to_string(total_elements) + ".");
    return NVPT_OK;
}

}  // extern "C"
