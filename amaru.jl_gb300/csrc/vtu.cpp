// VTU output: save_vtu (src/mesh/io.jl:167-274) with get_array_node! (:117-158) and the XML writer of
// src/tools/xml.jl:250-318, byte for byte, in ascii or, with compress=true, as appended raw zlib blocks.
//
// The file holds the model's points (coordinates as Float64 x 3), cells (0-based connectivity in
// Amaru's local node order, offsets and VTK cell types as Int32) and the caller's point and cell
// arrays in their order.  A float entry is "%20.10e" of the value rounded to Float32 (the Julia
// Printf output: NaN and Inf spelt as Julia does); an integer entry is the number and two spaces; a
// row is one line whose leading blanks become the element's indentation plus three.  Arrays come from
// host or device buffers; large arrays are formatted by host threads in row chunks, concatenated in
// order.  In the compressed form every DataArray is a self-closing element with format "appended" and
// the offset of its block; a block is the UInt64 header (1, n, n, compressed n) and the zlib stream
// (level 4, the zlib defaults of window 15 and memory level 8: the settings of the reference's
// ZlibCompressorStream) of the array's bytes in row order, blocks compressed by host threads in
// parallel and appended in order after "_" in <AppendedData encoding="raw">.  zlib is the system's
// libz.so.1, opened at the first compressed write.  Tags are columns the caller passes (tag-s1, tag-s2,
// tag), as update_output_data! leaves them in elem_data.
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "amr_internal.h"

namespace {

// the two zlib entry points the compressed form uses (zlib.h: compress2, compressBound)
using compress2_fn = int (*)(unsigned char *, unsigned long *, const unsigned char *, unsigned long, int);
using bound_fn = unsigned long (*)(unsigned long);
struct Zlib {
    compress2_fn compress2 = nullptr;
    bound_fn bound = nullptr;
};
const Zlib &zlib() {
    static Zlib z;
    static std::once_flag once;
    std::call_once(once, [] {
        void *h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) return;
        z.compress2 = reinterpret_cast<compress2_fn>(dlsym(h, "compress2"));
        z.bound = reinterpret_cast<bound_fn>(dlsym(h, "compressBound"));
        if (!z.compress2 || !z.bound) z.compress2 = nullptr;
    });
    if (!z.compress2) throw AmrError(AMR_EUNSUPPORTED, "compressed VTU output needs zlib (libz.so.1)");
    return z;
}

// VTK cell type of each shape (vtk_type in src/shape/*.jl, codes of src/shape/vtk.jl)
int vtk_type(int shape) {
    switch (shape) {
    case AMR_TRI3: return 5;
    case AMR_TRI6: return 22;
    case AMR_QUAD4: return 9;
    case AMR_QUAD8: return 23;
    case AMR_QUAD9: return 28;
    case AMR_TET4: return 10;
    case AMR_TET10: return 24;
    case AMR_HEX8: return 12;
    case AMR_HEX20: return 25;
    case AMR_LIN2: return 3;
    case AMR_LIN3: return 21;
    }
    return 0;
}

const char *type_name(int t) {
    switch (t) {
    case AMR_VTU_FLOAT64: return "Float64";
    case AMR_VTU_INT32: return "Int32";
    case AMR_VTU_INT64: return "Int64";
    case AMR_VTU_UINT64: return "UInt64";
    }
    return nullptr;
}

size_t elem_size(int t) { return t == AMR_VTU_INT32 ? 4 : 8; }

// "%20.10e" of Float32(v) as Julia's Printf writes it
void put_float(std::string &s, double v) {
    const float f = (float)v;
    char b[48];
    if (std::isnan(f)) std::snprintf(b, sizeof b, "%20s", "NaN");
    else if (std::isinf(f)) std::snprintf(b, sizeof b, "%20s", f > 0 ? "Inf" : "-Inf");
    else std::snprintf(b, sizeof b, "%20.10e", (double)f);
    s += b;
}

template <class T>
void put_int(std::string &s, T v) {
    s += std::to_string(v);
    s += "  ";
}

struct Array {
    std::string name;
    int type = AMR_VTU_FLOAT64, ncomp = 1;
    int64_t nrows = 0;
    std::vector<unsigned char> host;  // column-major nrows x ncomp
};

// the rows [r0, r1) of an array, each line indented and ended by a newline
void format_rows(const Array &a, int64_t r0, int64_t r1, const std::string &indent, std::string &out) {
    std::string row;
    for (int64_t i = r0; i < r1; i++) {
        row.clear();
        for (int c = 0; c < a.ncomp; c++) {
            const size_t at = (size_t)c * a.nrows + i;
            switch (a.type) {
            case AMR_VTU_FLOAT64: put_float(row, reinterpret_cast<const double *>(a.host.data())[at]); break;
            case AMR_VTU_INT32: put_int(row, reinterpret_cast<const int32_t *>(a.host.data())[at]); break;
            case AMR_VTU_INT64: put_int(row, reinterpret_cast<const int64_t *>(a.host.data())[at]); break;
            case AMR_VTU_UINT64: put_int(row, reinterpret_cast<const uint64_t *>(a.host.data())[at]); break;
            }
        }
        size_t k = 0;
        while (k < row.size() && row[k] == ' ') k++;
        out += indent;
        out.append(row, k, std::string::npos);
        out += '\n';
    }
}

// <DataArray ...> element at the given level (writenode for a DataArray with content)
void write_array(std::string &out, const Array &a, int level, int nthreads) {
    const std::string tab = "   ";
    std::string ind0, ind1;
    for (int i = 0; i < level; i++) ind0 += tab;
    ind1 = ind0 + tab;
    out += ind0 + "<DataArray type=\"" + type_name(a.type) + "\" Name=\"" + a.name + "\" NumberOfComponents=\"" +
           std::to_string(a.ncomp) + "\" format=\"ascii\">\n";
    const int64_t rows = a.nrows;
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads, rows / 4096));
    if (nt <= 1) {
        format_rows(a, 0, rows, ind1, out);
    } else {
        std::vector<std::string> parts(nt);
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++)
            th.emplace_back([&, t]() {
                const int64_t r0 = rows * t / nt, r1 = rows * (t + 1) / nt;
                parts[t].reserve((size_t)(r1 - r0) * (a.ncomp * 20 + ind1.size() + 1));
                format_rows(a, r0, r1, ind1, parts[t]);
            });
        for (auto &x : th) x.join();
        for (auto &p : parts) out += p;
    }
    out += ind0 + "</DataArray>\n";
}

// the array's block of the appended data: header and zlib stream of its row-major bytes
std::string compressed_block(const Array &a) {
    const size_t es = elem_size(a.type), n = a.host.size();
    std::vector<unsigned char> rows(n);
    for (int64_t i = 0; i < a.nrows; i++)
        for (int c = 0; c < a.ncomp; c++)
            std::memcpy(&rows[((size_t)i * a.ncomp + c) * es], &a.host[((size_t)c * a.nrows + i) * es], es);
    const Zlib &z = zlib();
    unsigned long zn = z.bound((unsigned long)n);
    std::string blk(32 + zn, '\0');
    const int rc = z.compress2(reinterpret_cast<unsigned char *>(&blk[32]), &zn, rows.data(), (unsigned long)n, 4);
    if (rc != 0) throw AmrError(AMR_EINVAL, "zlib compress2 failed (" + std::to_string(rc) + ")");
    const uint64_t head[4] = {1, (uint64_t)n, (uint64_t)n, (uint64_t)zn};
    std::memcpy(&blk[0], head, 32);
    blk.resize(32 + zn);
    return blk;
}

Array take(const amr_vtu_array &d, int64_t nrows) {
    if (!d.name || !type_name(d.type) || d.ncomp < 1 || (!d.data && nrows > 0))
        throw AmrError(AMR_EINVAL, "bad VTU array description");
    Array a;
    a.name = d.name;
    a.type = d.type;
    a.ncomp = d.ncomp;
    a.nrows = nrows;
    a.host.resize((size_t)nrows * d.ncomp * elem_size(d.type));
    if (a.host.empty()) return a;
    if (d.on_device) AMR_CUDA(cudaMemcpy(a.host.data(), d.data, a.host.size(), cudaMemcpyDeviceToHost));
    else std::memcpy(a.host.data(), d.data, a.host.size());
    return a;
}

}  // namespace

void amr_vtu_write(amr_model *m, const char *path, const amr_vtu_array *pd, int npd, const amr_vtu_array *cd,
                   int ncd, int nthreads, bool compress) {
    if (!path) throw AmrError(AMR_EINVAL, "null path");
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    const int64_t nn = m->nnodes, ne = m->nelems;
    // points and cells from the model, caller order
    Array pts;
    pts.name = "Points"; pts.type = AMR_VTU_FLOAT64; pts.ncomp = 3; pts.nrows = nn;
    pts.host.resize((size_t)nn * 3 * 8);
    double *P = reinterpret_cast<double *>(pts.host.data());
    for (int64_t i = 0; i < nn; i++)
        for (int c = 0; c < 3; c++) P[(size_t)c * nn + i] = m->h_coords[3 * i + c];
    Array conn, offs, types;
    conn.name = "connectivity"; conn.type = AMR_VTU_INT32;
    offs.name = "offsets"; offs.type = AMR_VTU_INT32; offs.nrows = ne;
    types.name = "types"; types.type = AMR_VTU_INT32; types.nrows = ne;
    std::vector<int32_t> cv, ov(ne), tv(ne);
    int32_t off = 0;
    for (int64_t e = 0; e < ne; e++) {
        const int64_t s = m->inv_perm[e];
        for (int64_t k = m->h_conn_ptr[s]; k < m->h_conn_ptr[s + 1]; k++) cv.push_back(m->h_conn[k]);
        off += (int32_t)(m->h_conn_ptr[s + 1] - m->h_conn_ptr[s]);
        ov[e] = off;
        tv[e] = vtk_type(m->h_shape[s]);
    }
    conn.nrows = (int64_t)cv.size();
    auto bytes = [](const std::vector<int32_t> &v) {
        return std::vector<unsigned char>((const unsigned char *)v.data(), (const unsigned char *)(v.data() + v.size()));
    };
    conn.host = bytes(cv); offs.host = bytes(ov); types.host = bytes(tv);
    std::vector<Array> pa, ca;
    for (int i = 0; i < npd; i++) pa.push_back(take(pd[i], nn));
    for (int i = 0; i < ncd; i++) ca.push_back(take(cd[i], ne));
    // compressed form: every array's block, compressed in parallel, offsets in document order
    std::vector<const Array *> order{&pts, &conn, &offs, &types};
    for (const Array &a : pa)
        if (a.nrows * a.ncomp > 0) order.push_back(&a);
    for (const Array &a : ca)
        if (a.nrows * a.ncomp > 0) order.push_back(&a);
    std::vector<std::string> blocks;
    std::vector<size_t> offset;
    if (compress) {
        zlib();
        blocks.resize(order.size());
        std::vector<std::thread> th;
        const int nt = std::max(1, std::min<int>(nthreads, (int)order.size()));
        for (int t = 0; t < nt; t++)
            th.emplace_back([&, t]() {
                for (size_t i = t; i < order.size(); i += nt) blocks[i] = compressed_block(*order[i]);
            });
        for (auto &x : th) x.join();
        size_t o = 0;
        for (auto &b : blocks) { offset.push_back(o); o += b.size(); }
    }
    size_t next = 0;  // index into order of the next array written
    auto array = [&](std::string &out, const Array &a) {
        if (!compress) {
            write_array(out, a, 4, nthreads);
            return;
        }
        out += std::string("            <DataArray type=\"") + type_name(a.type) + "\" Name=\"" + a.name +
               "\" NumberOfComponents=\"" + std::to_string(a.ncomp) + "\" format=\"appended\" offset=\"" +
               std::to_string(offset[next]) + "\"/>\n";
        next++;
    };
    // document (xml.jl save + writenode)
    std::string out;
    if (!compress) out.reserve((size_t)nn * (3 + 16) * 22 + (size_t)conn.nrows * 14);
    out += "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n";
    out += "<!-- File generated by Amaru Finite Element Code -->\n";
    out += "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\" "
           "compressor=\"vtkZLibDataCompressor\">\n";
    out += "   <UnstructuredGrid>\n";
    out += "      <Piece NumberOfPoints=\"" + std::to_string(nn) + "\" NumberOfCells=\"" + std::to_string(ne) + "\">\n";
    out += "         <Points>\n";
    array(out, pts);
    out += "         </Points>\n";
    out += "         <Cells>\n";
    array(out, conn);
    array(out, offs);
    array(out, types);
    out += "         </Cells>\n";
    auto section = [&](const char *tag, const std::vector<Array> &arrs) {
        if (arrs.empty()) return;  // no data: no element (save_vtu's has_node_data / has_elem_data)
        bool any = false;
        for (const Array &a : arrs) any |= a.nrows * a.ncomp > 0;
        if (!any) {  // an element without children or content closes itself (writenode)
            out += std::string("         <") + tag + "/>\n";
            return;
        }
        out += std::string("         <") + tag + ">\n";
        for (const Array &a : arrs)
            if (a.nrows * a.ncomp > 0) array(out, a);  // empty arrays are skipped
        out += std::string("         </") + tag + ">\n";
    };
    section("PointData", pa);
    section("CellData", ca);
    out += "      </Piece>\n";
    out += "   </UnstructuredGrid>\n";
    FILE *f = std::fopen(path, "wb");
    if (!f) throw AmrError(AMR_EINVAL, std::string("cannot open ") + path);
    bool ok = true;
    auto put = [&](const std::string &x) { ok = ok && std::fwrite(x.data(), 1, x.size(), f) == x.size(); };
    if (compress) {
        out += "   <AppendedData encoding=\"raw\">\n_";
        put(out);
        for (auto &b : blocks) put(b);
        put("\n   </AppendedData>\n</VTKFile>\n");
    } else {
        out += "</VTKFile>\n";
        put(out);
    }
    const int rc = std::fclose(f);
    if (!ok || rc != 0) throw AmrError(AMR_EINVAL, std::string("write failed: ") + path);
}
