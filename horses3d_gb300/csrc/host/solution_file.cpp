// HORSES3D solution files (.hsol), io/SolutionFile.f90:1-628 and HexMesh_SaveSolution /
// HexMesh_LoadSolution (HexMesh.f90:3376-3555, 4708-): a stream-access binary file with
//   byte 0    file name (128 characters, the name given at creation)
//   byte 128  file type (int32: 2 solution, 3 solution and gradients, ...)
//   byte 132  node type (int32: 1 Gauss, 2 Gauss-Lobatto)
//   byte 136  number of elements (int32)
//   byte 140  iteration (int32)
//   byte 144  time (float64)
//   byte 152  reference values gamma, R, V, rho, T, Mach (6 x float64)
//   byte 200  88 (beginning of data)
//   byte 204  per element: 4 (int32 rank), NCONS, Nx+1, Ny+1, Nz+1 (int32), Q(1:5,0:Nx,0:Ny,0:Nz)
//             (float64, column-major); gradient files (types 3, 10) then add U_x, U_y, U_z (5 values
//             per node each); sensor files (types 9, 10) end the record with the element's sensor
//             value (float64), HexMesh.f90:3522-3525, 4832
//   end       99 (int32)
// Little-endian, as the reference writes it on the platforms it runs on.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "horses3d_gb300.h"
#include "status.hpp"

namespace {

constexpr int kBeginData = 88;
constexpr int kEndOfFile = 99;
constexpr long kHeaderBytes = 204;

struct File {
    std::FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

bool read_at(std::FILE* f, long pos, void* dst, size_t n) {
    return std::fseek(f, pos, SEEK_SET) == 0 && std::fread(dst, 1, n, f) == n;
}

}  // namespace

extern "C" {

int h3d_read_solution_header(const char* path, h3d_solution_header* h) {
    if (!path || !h) return h3d::fail(DG_ERR_INVALID, "null argument");
    File fl;
    fl.f = std::fopen(path, "rb");
    if (!fl.f) return h3d::fail(DG_ERR_IO, std::string("cannot open ") + path);
    char name[129] = {};
    int32_t ints[4];
    double t, refs[6];
    int32_t term;
    if (!read_at(fl.f, 0, name, 128) || !read_at(fl.f, 128, ints, 16) || !read_at(fl.f, 144, &t, 8) ||
        !read_at(fl.f, 152, refs, 48) || !read_at(fl.f, 200, &term, 4))
        return h3d::fail(DG_ERR_IO, std::string(path) + ": truncated solution file header");
    if (term != kBeginData) return h3d::fail(DG_ERR_IO, std::string(path) + ": wrong beginning data specifier");
    std::memset(h, 0, sizeof(*h));
    std::memcpy(h->name, name, 128);
    h->file_type = ints[0];
    h->node_type = ints[1];
    h->n_elements = ints[2];
    h->iteration = ints[3];
    h->time = t;
    for (int k = 0; k < 6; ++k) h->refs[k] = refs[k];
    return DG_OK;
}

int h3d_read_solution(const char* path, int32_t n_elements, const int32_t* orders, double* q, double* gradients) {
    if (!path || !orders || !q) return h3d::fail(DG_ERR_INVALID, "null argument");
    h3d_solution_header h;
    int rc = h3d_read_solution_header(path, &h);
    if (rc) return rc;
    if (h.n_elements != n_elements)
        return h3d::fail(DG_ERR_INVALID, std::string(path) + ": the file holds " + std::to_string(h.n_elements) +
                                             " elements, the mesh " + std::to_string(n_elements));
    // The file types HexMesh_LoadSolution restarts from (HexMesh.f90:4744-4780): solution (2),
    // solution and gradients (3), either with the per-element sensor value (9, 10).
    if (h.file_type != 2 && h.file_type != 3 && h.file_type != 9 && h.file_type != 10)
        return h3d::fail(DG_ERR_INVALID, std::string(path) + ": file type " + std::to_string(h.file_type) +
                                             " is not a solution file (2, 3, 9 or 10)");
    const bool has_grad = h.file_type == 3 || h.file_type == 10;
    const bool has_sensor = h.file_type == 9 || h.file_type == 10;
    if (gradients && !has_grad) return h3d::fail(DG_ERR_INVALID, std::string(path) + ": the file holds no gradients");
    const int padding = has_grad ? 20 : 5;  // values per node: Q (5) [+ U_x, U_y, U_z (5 each)]
    File fl;
    fl.f = std::fopen(path, "rb");
    if (!fl.f) return h3d::fail(DG_ERR_IO, std::string("cannot open ") + path);
    long pos = kHeaderBytes;
    int64_t off = 0;
    for (int e = 0; e < n_elements; ++e) {
        int32_t rec[5];
        if (!read_at(fl.f, pos, rec, 20)) return h3d::fail(DG_ERR_IO, std::string(path) + ": truncated element record");
        const int px = orders[3 * e] + 1, py = orders[3 * e + 1] + 1, pz = orders[3 * e + 2] + 1;
        if (rec[0] != 4 || rec[1] != 5 || rec[2] != px || rec[3] != py || rec[4] != pz)
            return h3d::fail(DG_ERR_INVALID, std::string(path) + ": element " + std::to_string(e) +
                                                 " has other polynomial orders than the mesh");
        const size_t np = static_cast<size_t>(px) * py * pz;
        if (std::fread(q + 5 * off, sizeof(double), 5 * np, fl.f) != 5 * np)
            return h3d::fail(DG_ERR_IO, std::string(path) + ": truncated element data");
        if (gradients) {
            for (int d = 0; d < 3; ++d)
                if (std::fread(gradients + 15 * off + 5 * np * d, sizeof(double), 5 * np, fl.f) != 5 * np)
                    return h3d::fail(DG_ERR_IO, std::string(path) + ": truncated gradient data");
        }
        pos += 20 + static_cast<long>(padding) * static_cast<long>(np) * 8 + (has_sensor ? 8 : 0);
        off += static_cast<int64_t>(np);
    }
    return DG_OK;
}

int h3d_write_solution(const char* path, const h3d_solution_header* h, const int32_t* orders, const double* q,
                       const double* gradients) {
    if (!path || !h || !orders || !q) return h3d::fail(DG_ERR_INVALID, "null argument");
    const bool has_grad = gradients != nullptr;
    if (has_grad != (h->file_type == 3)) return h3d::fail(DG_ERR_INVALID, "file type 3 is the one with gradients, 2 without");
    File fl;
    fl.f = std::fopen(path, "wb");
    if (!fl.f) return h3d::fail(DG_ERR_IO, std::string("cannot create ") + path);
    char name[128] = {};
    std::memcpy(name, h->name, 128);
    const int32_t ints[4] = {h->file_type, h->node_type, h->n_elements, h->iteration};
    const int32_t begin = kBeginData;
    bool ok = std::fwrite(name, 1, 128, fl.f) == 128 && std::fwrite(ints, 4, 4, fl.f) == 4 &&
              std::fwrite(&h->time, 8, 1, fl.f) == 1 && std::fwrite(h->refs, 8, 6, fl.f) == 6 &&
              std::fwrite(&begin, 4, 1, fl.f) == 1;
    int64_t off = 0;
    for (int e = 0; ok && e < h->n_elements; ++e) {
        const int px = orders[3 * e] + 1, py = orders[3 * e + 1] + 1, pz = orders[3 * e + 2] + 1;
        const int32_t rec[5] = {4, 5, px, py, pz};
        const size_t np = static_cast<size_t>(px) * py * pz;
        ok = std::fwrite(rec, 4, 5, fl.f) == 5 && std::fwrite(q + 5 * off, 8, 5 * np, fl.f) == 5 * np;
        for (int d = 0; ok && has_grad && d < 3; ++d)
            ok = std::fwrite(gradients + 15 * off + 5 * np * d, 8, 5 * np, fl.f) == 5 * np;
        off += static_cast<int64_t>(np);
    }
    const int32_t end = kEndOfFile;
    ok = ok && std::fwrite(&end, 4, 1, fl.f) == 1;
    if (!ok) return h3d::fail(DG_ERR_IO, std::string(path) + ": write failed");
    return DG_OK;
}

}  // extern "C"
