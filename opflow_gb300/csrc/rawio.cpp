// Field snapshots in OpFlow's raw binary format (Utils::RawBinaryOStream / RawBinaryIStream,
// src/Utils/Writers/RawBinaryStream.hpp:80-224), for checkpoint and restore.  One file
// <dir>/<name>_<count>.cart per written field, little-endian, laid out as the reference writes it:
//   int name length, the name's characters, int dim, int rank count (1: one process per field),
//   double time,
//   dim x (int start, int end)   mesh range,
//   the mesh's node coordinates x(d, j) for j in the mesh range, dim after dim,
//   dim x (int start, int end)   the field's accessible range,
//   dim x (int start, int end)   the field's local range,
//   the values over the local range, x fastest (float64).
// Reading checks the name (a mismatch is not an error, as in the reference), dim, rank count, mesh
// range and coordinates, accessible and local ranges, then stores the values and refreshes the padding.
#include "internal.h"

#include <cstdio>
#include <string>
#include <vector>

namespace opg {
namespace {

std::string cart_path(const char* dir, const char* name, int count) {
    std::string p = dir && *dir ? std::string(dir) : std::string(".");
    return p + "/" + name + "_" + std::to_string(count) + ".cart";
}

// the local range over the field's data array, x fastest
template <typename F>
void for_local(const opflow_field_info& I, F&& fn) {
    const int D = I.ndim;
    int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    for (int d = 0; d < D; ++d) { lo[d] = I.local[d][0]; hi[d] = I.local[d][1]; }
    for (int k = lo[2]; k < hi[2]; ++k)
        for (int j = lo[1]; j < hi[1]; ++j)
            for (int i = lo[0]; i < hi[0]; ++i) {
                const int idx[3] = {i, j, k};
                long long o = 0, stride = 1;
                for (int d = 0; d < D; ++d) {
                    o += (long long) (idx[d] - I.data_offset[d]) * stride;
                    stride *= I.data_dims[d];
                }
                fn(o);
            }
}

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

}  // namespace
}  // namespace opg

using namespace opg;

extern "C" {

int opflow_field_write_raw(opflow_field f, const char* dir, const char* name, int count, double time) {
    if (!f || !name) return fail(OPFLOW_E_INVALID, "null argument");
    const opflow_field_info& I = f->info;
    const MeshDev* m = f->mesh;
    std::vector<double> data(I.count);
    OPG_TRY(opflow_field_download(f, data.data(), data.size()));
    const std::string path = cart_path(dir, name, count);
    File out;
    out.f = std::fopen(path.c_str(), "wb");
    if (!out.f) return fail(OPFLOW_E_INVALID, "cannot open %s for writing", path.c_str());
    bool ok = true;
    auto w = [&](const void* p, size_t sz, size_t n) { ok = ok && std::fwrite(p, sz, n, out.f) == n; };
    const int name_len = (int) std::string(name).size(), dim = I.ndim, nproc = 1;
    w(&name_len, sizeof(int), 1);
    w(name, 1, (size_t) name_len);
    w(&dim, sizeof(int), 1);
    w(&nproc, sizeof(int), 1);
    w(&time, sizeof(double), 1);
    for (int d = 0; d < dim; ++d) {
        const int s = m->es[d] + m->pad, e = m->es[d] + m->n[d] - m->pad;
        w(&s, sizeof(int), 1);
        w(&e, sizeof(int), 1);
    }
    for (int d = 0; d < dim; ++d) w(m->hx[d].data() + m->pad, sizeof(double), (size_t) (m->n[d] - 2 * m->pad));
    for (int d = 0; d < dim; ++d) w(I.accessible[d], sizeof(int), 2);
    for (int d = 0; d < dim; ++d) w(I.local[d], sizeof(int), 2);
    std::vector<double> vals;
    for_local(I, [&](long long o) { vals.push_back(data[o]); });
    w(vals.data(), sizeof(double), vals.size());
    if (!ok) return fail(OPFLOW_E_INVALID, "short write to %s", path.c_str());
    return OPFLOW_OK;
}

int opflow_field_read_raw(opflow_field f, const char* dir, const char* name, int count, double* time_out) {
    if (!f || !name) return fail(OPFLOW_E_INVALID, "null argument");
    const opflow_field_info& I = f->info;
    const MeshDev* m = f->mesh;
    const std::string path = cart_path(dir, name, count);
    File in;
    in.f = std::fopen(path.c_str(), "rb");
    if (!in.f) return fail(OPFLOW_E_INVALID, "cannot open %s", path.c_str());
    bool ok = true;
    auto r = [&](void* p, size_t sz, size_t n) { ok = ok && std::fread(p, sz, n, in.f) == n; };
    int name_len = 0;
    r(&name_len, sizeof(int), 1);
    if (!ok || name_len < 0 || name_len > (1 << 20)) return fail(OPFLOW_E_INVALID, "%s: bad header", path.c_str());
    std::string fname((size_t) name_len, '\0');
    r(&fname[0], 1, (size_t) name_len);
    int dim = 0, nproc = 0;
    r(&dim, sizeof(int), 1);
    r(&nproc, sizeof(int), 1);
    if (!ok || dim != I.ndim) return fail(OPFLOW_E_INVALID, "%s: dim mismatch %d != %d", path.c_str(), dim, I.ndim);
    if (nproc != 1) return fail(OPFLOW_E_INVALID, "%s: data set written by %d ranks, read by 1", path.c_str(), nproc);
    double t = 0.;
    r(&t, sizeof(double), 1);
    for (int d = 0; d < dim; ++d) {
        int se[2];
        r(se, sizeof(int), 2);
        if (!ok || se[0] != m->es[d] + m->pad || se[1] != m->es[d] + m->n[d] - m->pad)
            return fail(OPFLOW_E_INVALID, "%s: mesh range mismatch along dim %d", path.c_str(), d);
    }
    for (int d = 0; d < dim; ++d) {
        std::vector<double> xs((size_t) (m->n[d] - 2 * m->pad));
        r(xs.data(), sizeof(double), xs.size());
        for (size_t j = 0; ok && j < xs.size(); ++j)
            if (xs[j] != m->hx[d][j + m->pad]) return fail(OPFLOW_E_INVALID, "%s: mesh coordinate mismatch at x[%d][%zu]", path.c_str(), d, j);
    }
    for (int pass = 0; pass < 2; ++pass)
        for (int d = 0; d < dim; ++d) {
            int se[2];
            r(se, sizeof(int), 2);
            const int* want = pass == 0 ? I.accessible[d] : I.local[d];
            if (!ok || se[0] != want[0] || se[1] != want[1])
                return fail(OPFLOW_E_INVALID, "%s: field %s range mismatch along dim %d", path.c_str(), pass == 0 ? "accessible" : "local", d);
        }
    std::vector<double> data(I.count);
    OPG_TRY(opflow_field_download(f, data.data(), data.size()));
    for_local(I, [&](long long o) { r(&data[o], sizeof(double), 1); });
    if (!ok) return fail(OPFLOW_E_INVALID, "%s: file ends before the field's values", path.c_str());
    OPG_TRY(opflow_field_upload(f, data.data(), data.size()));
    OPG_TRY(opflow_field_update_padding(f));
    if (time_out) *time_out = t;
    return OPFLOW_OK;
}

}  // extern "C"
