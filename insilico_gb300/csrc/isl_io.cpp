// Mesh and field I/O fast paths, with the reference's text layouts:
//  * SMF meshes: base/io/smf/Reader.hpp:98-313 and Writer.hpp:60-140; the
//    format is described in base/io/smf/smf.hpp;
//  * legacy VTK unstructured grids with point and cell data:
//    base/io/vtk/LegacyWriter.hpp:86-290 with the value layout of
//    base/io/raw/ascii.hpp:24-178 and the cell types of
//    base/io/vtk/CellTraits.hpp.
// A file is read whole, cut at line boundaries into one chunk per host
// thread, and every chunk is converted by its own thread: std::from_chars
// (correctly rounded, as the reference's istream >> double) for reading, and
// "%g" (what an ostream with default precision prints) for writing.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "isl_internal.h"

namespace {

bool read_file(const char* path, std::string& out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out.resize(n > 0 ? (size_t)n : 0);
    const size_t got = n > 0 ? std::fread(&out[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == out.size();
}

unsigned nthreads() {
    const unsigned h = std::thread::hardware_concurrency();
    return std::max(1u, std::min(h ? h : 1u, 64u));
}

// run fn(lo, hi) on [0, n) split into one range per thread
template <typename F>
void parallel_ranges(int64_t n, F fn) {
    const int64_t nt = std::min<int64_t>(nthreads(), std::max<int64_t>(1, n / 4096));
    if (nt <= 1) { fn(0, n); return; }
    std::vector<std::thread> th;
    for (int64_t t = 0; t < nt; ++t) th.emplace_back(fn, n * t / nt, n * (t + 1) / nt);
    for (auto& x : th) x.join();
}

const char* skip_ws(const char* p, const char* end) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
    return p;
}

bool parse_double(const char*& p, const char* end, double& v) {
    p = skip_ws(p, end);
    if (p < end && *p == '+') ++p;
    auto r = std::from_chars(p, end, v);
    if (r.ec != std::errc()) return false;
    p = r.ptr;
    return true;
}

bool parse_int(const char*& p, const char* end, int64_t& v) {
    p = skip_ws(p, end);
    if (p < end && *p == '+') ++p;
    auto r = std::from_chars(p, end, v);
    if (r.ec != std::errc()) return false;
    p = r.ptr;
    return true;
}

// the starts of the next n lines from position pos (a line = up to '\n')
bool line_starts(const std::string& s, size_t pos, int64_t n, std::vector<size_t>& starts, size_t& after) {
    // every line holds at least one byte: a count above the bytes left is
    // rejected before anything is sized by it
    if (n < 0 || pos > s.size() || (uint64_t)n > (uint64_t)(s.size() - pos)) return false;
    starts.resize((size_t)n + 1);
    size_t p = pos;
    for (int64_t i = 0; i < n; ++i) {
        if (p >= s.size()) return false;
        starts[(size_t)i] = p;
        const void* nl = std::memchr(s.data() + p, '\n', s.size() - p);
        p = nl ? (size_t)((const char*)nl - s.data()) + 1 : s.size();
    }
    starts[(size_t)n] = p;
    after = p;
    return true;
}

// per line: the first k numbers (the rest of the line is ignored, as the
// reader's ignore(..., '\n'))
template <typename T, typename P>
bool parse_lines(const std::string& s, const std::vector<size_t>& starts, int64_t n, int k, T* out, P parse) {
    std::atomic<bool> fail{false};
    parallel_ranges(n, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi && !fail.load(std::memory_order_relaxed); ++i) {
            const char* p = s.data() + starts[(size_t)i];
            const char* end = s.data() + starts[(size_t)i + 1];
            for (int j = 0; j < k; ++j)
                if (!parse(p, end, out[i * k + j])) { fail = true; break; }
        }
    });
    return !fail;
}

std::string lower(std::string x) {
    for (auto& ch : x) ch = (char)std::tolower((unsigned char)ch);
    return x;
}

const char* shape_name(int shape) {
    return shape == ISL_QUAD ? "quadrilateral" : shape == ISL_HEX ? "hexahedron" : "tetrahedron";
}
int shape_nodes(int shape) { return shape == ISL_HEX ? 8 : 4; }
int shape_dim(int shape) { return shape == ISL_QUAD ? 2 : 3; }

// one line of the header: "!" descriptor value (base/io/smf/Reader.hpp:209-251)
void header_tokens(const std::string& line, std::vector<std::string>& tok) {
    tok.clear();
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && line[i] == ' ') ++i;
        size_t j = i;
        while (j < line.size() && line[j] != ' ') ++j;
        if (j > i) tok.push_back(line.substr(i, j - i));
        i = j;
    }
}

// "%g" into buf, as an ostream with default precision writes a double
inline int fmt_g(char* buf, double v) { return std::snprintf(buf, 32, "%g", v); }

// format n records in parallel (each into its own chunk buffer) and write the
// chunks in order
template <typename F>
bool write_records(FILE* f, int64_t n, F fmt) {
    const int64_t nt = std::min<int64_t>(nthreads(), std::max<int64_t>(1, n / 4096));
    std::vector<std::string> parts((size_t)nt);
    auto work = [&](int64_t t) {
        std::string& out = parts[(size_t)t];
        const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        out.reserve((size_t)(hi - lo) * 32);
        for (int64_t i = lo; i < hi; ++i) fmt(i, out);
    };
    if (nt <= 1) work(0);
    else {
        std::vector<std::thread> th;
        for (int64_t t = 0; t < nt; ++t) th.emplace_back(work, t);
        for (auto& x : th) x.join();
    }
    for (auto& p : parts)
        if (!p.empty() && std::fwrite(p.data(), 1, p.size(), f) != p.size()) return false;
    return true;
}

void put_g(std::string& out, double v) {
    char b[32];
    const int k = fmt_g(b, v);
    out.append(b, (size_t)k);
}

void put_i(std::string& out, int64_t v) {
    char b[24];
    auto r = std::to_chars(b, b + sizeof b, v);
    out.append(b, (size_t)(r.ptr - b));
}

// nodal coordinates as base/io/raw/ascii.hpp:92-102: dim values, each with a
// trailing blank, padded with "0 " to three
void put_node(std::string& out, const double* x, int dim) {
    for (int d = 0; d < dim; ++d) { put_g(out, x[d]); out += ' '; }
    for (int d = dim; d < 3; ++d) out += "0 ";
    out += '\n';
}

}  // namespace

extern "C" {

int isl_mesh_read_smf(isl_ctx* c, const char* path, int shape) {
    ISL_TRY
    if (!c || !path) return ISL_ERR_ARG;
    if (!(shape == ISL_QUAD || shape == ISL_TET || shape == ISL_HEX)) ISL_FAIL(c, ISL_ERR_ARG, "unsupported shape");
    std::string s;
    if (!read_file(path, s)) ISL_FAIL(c, ISL_ERR_ARG, std::string("cannot read ") + path);
    size_t pos = 0;
    auto line_at = [&](size_t p) {
        const size_t e = s.find('\n', p);
        return s.substr(p, (e == std::string::npos ? s.size() : e) - p);
    };
    auto next_line = [&](size_t p) {
        const size_t e = s.find('\n', p);
        return e == std::string::npos ? s.size() : e + 1;
    };
    // header (Reader.hpp:187-262): comments, then "!" lines, then comments
    while (pos < s.size() && s[pos] == '#') pos = next_line(pos);
    bool found_shape = false, found_num = false;
    std::string ext_nodes, ext_elems;
    std::vector<std::string> tok;
    while (pos < s.size() && s[pos] == '!') {
        std::string line = line_at(pos + 1);
        if (!line.empty() && line.back() == '\r') line.pop_back();
        pos = next_line(pos);
        header_tokens(line, tok);
        if (tok.empty()) continue;
        const std::string& d = tok[0];
        const std::string v = tok.size() > 1 ? tok[1] : std::string();
        if (d.find("elementShape") != std::string::npos) {
            found_shape = true;
            if (lower(v).find(shape_name(shape)) == std::string::npos)
                ISL_FAIL(c, ISL_ERR_ARG, "Smf file has unexpected shape value: " + v + " != " + shape_name(shape));
        } else if (d.find("elementNumPoints") != std::string::npos) {
            found_num = true;
            int64_t k = -1;
            const char* p = v.data();
            if (!parse_int(p, v.data() + v.size(), k) || k != shape_nodes(shape))
                ISL_FAIL(c, ISL_ERR_ARG, "Smf file has unexpected number of element nodes: " + v);
        } else if (d.find("externalNodes") != std::string::npos) {
            ext_nodes = v;
        } else if (d.find("externalElements") != std::string::npos) {
            ext_elems = v;
        }
    }
    while (pos < s.size() && s[pos] == '#') pos = next_line(pos);
    if (!(found_shape && found_num)) ISL_FAIL(c, ISL_ERR_ARG, "Smf header is invalid");
    // "nNodes nElements", rest of the line ignored (Reader.hpp:166-172)
    int64_t nn = 0, ne = 0;
    {
        const char* p = s.data() + pos;
        const char* end = s.data() + s.size();
        if (!parse_int(p, end, nn) || !parse_int(p, end, ne) || nn <= 0 || ne <= 0)
            ISL_FAIL(c, ISL_ERR_ARG, "Smf: bad node / element counts");
        pos = next_line((size_t)(p - s.data()));
    }
    const int dim = shape_dim(shape), nv = shape_nodes(shape);
    std::vector<double> X;
    std::vector<int64_t> conn;
    std::vector<size_t> starts;
    size_t after = 0;
    // nodes: the first dim numbers of each line (raw/ascii.hpp:108-119)
    {
        std::string ext;
        const std::string* src = &s;
        size_t p0 = pos;
        if (!ext_nodes.empty()) {
            if (!read_file(ext_nodes.c_str(), ext)) ISL_FAIL(c, ISL_ERR_ARG, "Failed to open " + ext_nodes);
            src = &ext;
            p0 = 0;
        }
        if (!line_starts(*src, p0, nn, starts, after)) ISL_FAIL(c, ISL_ERR_ARG, "Smf: fewer node lines than announced");
        X.resize((size_t)nn * dim);
        if (!parse_lines(*src, starts, nn, dim, X.data(), parse_double)) ISL_FAIL(c, ISL_ERR_ARG, "Smf: bad coordinate");
        if (ext_nodes.empty()) pos = after;
    }
    // elements: the node indices of each line, 0-based (raw/ascii.hpp:146-165)
    {
        std::string ext;
        const std::string* src = &s;
        size_t p0 = pos;
        if (!ext_elems.empty()) {
            if (!read_file(ext_elems.c_str(), ext)) ISL_FAIL(c, ISL_ERR_ARG, "Failed to open " + ext_elems);
            src = &ext;
            p0 = 0;
        }
        if (!line_starts(*src, p0, ne, starts, after)) ISL_FAIL(c, ISL_ERR_ARG, "Smf: fewer element lines than announced");
        conn.resize((size_t)ne * nv);
        if (!parse_lines(*src, starts, ne, nv, conn.data(), parse_int)) ISL_FAIL(c, ISL_ERR_ARG, "Smf: bad connectivity");
    }
    return isl_mesh_upload(c, shape, dim, nn, X.data(), ne, conn.data());
    ISL_CATCH(c)
}

int isl_mesh_get(isl_ctx* c, int64_t* n_nodes, int64_t* n_elem, double* X, int64_t* conn) {
    ISL_TRY
    if (!c || !c->nelem) return ISL_ERR_ARG;
    if (n_nodes) *n_nodes = c->nnodes;
    if (n_elem) *n_elem = c->nelem;
    if (X) std::copy(c->hX.begin(), c->hX.end(), X);
    if (conn) std::copy(c->hconn.begin(), c->hconn.end(), conn);
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_mesh_write_smf(isl_ctx* c, const char* path) {
    ISL_TRY
    if (!c || !path || !c->nelem) return ISL_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) ISL_FAIL(c, ISL_ERR_ARG, std::string("cannot write ") + path);
    const int dim = c->dim, nv = c->ngeom;
    std::string head = std::string("! elementShape ") + shape_name(c->shape) + "\n! elementNumPoints " +
                       std::to_string(nv) + "\n" + std::to_string(c->nnodes) + "  " + std::to_string(c->nelem) + "\n";
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
    ok = ok && write_records(f, c->nnodes, [&](int64_t i, std::string& out) { put_node(out, &c->hX[(size_t)i * dim], dim); });
    ok = ok && write_records(f, c->nelem, [&](int64_t e, std::string& out) {
        for (int v = 0; v < nv; ++v) { put_i(out, c->hconn[(size_t)e * nv + v]); out += ' '; }
        out += '\n';
    });
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) ISL_FAIL(c, ISL_ERR_ARG, std::string("write failed: ") + path);
    return ISL_OK;
    ISL_CATCH(c)
}

int isl_write_vtk(isl_ctx* c, const char* path, const char* point_name, const char* cell_name, int cell_rows,
                  int cell_cols, const double* cell_values) {
    ISL_TRY
    if (!c || !path || !c->nelem) return ISL_ERR_ARG;
    if (point_name && !c->fedeg) ISL_FAIL(c, ISL_ERR_ARG, "vtk: point data needs a field");
    if (cell_name && (!cell_values || cell_rows < 0 || cell_cols < 0 || cell_rows > 3 || cell_cols > 3 ||
                      (cell_rows == 0) != (cell_cols == 0)))
        ISL_FAIL(c, ISL_ERR_ARG, "vtk: cell data needs values of 0x0 (plain scalars) or r x c (r, c <= 3) per cell");
    // nodal values: the field at the geometry nodes.  For Lagrange elements the
    // value at a vertex is the vertex DOF's value (the shape functions are 0 or
    // 1 there), which is what evaluateFieldAtNodes interpolates
    // (base/post/evaluateAtNodes.hpp:103-175).
    std::vector<double> nodal;
    const int nc = c->ncomp;
    if (point_name) {
        std::vector<double> u((size_t)c->ndofobj * nc);
        if (c->device >= 0) {
            cudaSetDevice(c->device);
            ISL_CHECK_CUDA(c, cudaMemcpyAsync(u.data(), c->du.p, u.size() * 8, cudaMemcpyDeviceToHost, c->stream));
            ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
        } else {
            if (c->hu.size() != u.size()) ISL_FAIL(c, ISL_ERR_ARG, "vtk: no field values");
            u = c->hu;
        }
        nodal.assign((size_t)c->nnodes * nc, 0.0);
        for (int64_t e = 0; e < c->nelem; ++e)
            for (int v = 0; v < c->ngeom; ++v) {
                const int64_t node = c->hconn[(size_t)e * c->ngeom + v];
                const int64_t o = c->hedof[(size_t)e * c->nfun + v];
                for (int k = 0; k < nc; ++k) nodal[(size_t)node * nc + k] = u[(size_t)o * nc + k];
            }
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) ISL_FAIL(c, ISL_ERR_ARG, std::string("cannot write ") + path);
    const int dim = c->dim, nv = c->ngeom;
    const int ctype = c->shape == ISL_QUAD ? 9 : c->shape == ISL_HEX ? 12 : 10;  // CellTraits.hpp
    auto puts_ = [&](const std::string& t) { return std::fwrite(t.data(), 1, t.size(), f) == t.size(); };
    bool ok = puts_("# vtk DataFile Version 2.0\nGenerated by inSilico's base::io::vtk::LegacyWriter\nASCII\n");
    ok = ok && puts_("DATASET UNSTRUCTURED_GRID\nPOINTS " + std::to_string(c->nnodes) + " float\n");
    ok = ok && write_records(f, c->nnodes, [&](int64_t i, std::string& out) { put_node(out, &c->hX[(size_t)i * dim], dim); });
    ok = ok && puts_("CELLS " + std::to_string(c->nelem) + " " + std::to_string(c->nelem * (nv + 1)) + "\n");
    ok = ok && write_records(f, c->nelem, [&](int64_t e, std::string& out) {
        put_i(out, nv);
        out += ' ';
        for (int v = 0; v < nv; ++v) { put_i(out, c->hconn[(size_t)e * nv + v]); out += ' '; }
        out += '\n';
    });
    ok = ok && puts_("CELL_TYPES " + std::to_string(c->nelem) + "\n");
    ok = ok && write_records(f, c->nelem, [&](int64_t, std::string& out) { put_i(out, ctype); out += '\n'; });
    // a vector value: its rows, each value with a blank; 2-D rows and columns
    // padded with zeros to three (raw/ascii.hpp:24-49)
    auto put_mat = [](std::string& out, const double* v, int rows, int cols) {
        for (int r = 0; r < rows; ++r) {
            for (int k = 0; k < cols; ++k) { put_g(out, v[r * cols + k]); out += ' '; }
            if (cols == 2) out += "0 ";
        }
        if (rows == 2) {
            for (int k = 0; k < cols; ++k) out += "0 ";
            if (cols == 2) out += "0 ";
        }
    };
    auto kind = [](int size) { return size == 1 ? "SCALARS" : (size == 4 || size == 9) ? "TENSORS" : "VECTORS"; };
    if (point_name) {
        ok = ok && puts_("POINT_DATA " + std::to_string(c->nnodes) + "\n");
        ok = ok && puts_(std::string(kind(nc)) + " " + point_name + " float \n");
        if (nc == 1) ok = ok && puts_("LOOKUP_TABLE default \n");
        ok = ok && write_records(f, c->nnodes, [&](int64_t i, std::string& out) {
            put_mat(out, &nodal[(size_t)i * nc], nc, 1);
            out += '\n';
        });
    }
    if (cell_name) {
        const int size = cell_rows * cell_cols;
        ok = ok && puts_("CELL_DATA " + std::to_string(c->nelem) + "\n");
        ok = ok && puts_(std::string(size == 0 ? "SCALARS" : kind(size)) + " " + cell_name + " float \n");
        if (size <= 1) ok = ok && puts_("LOOKUP_TABLE default \n");
        ok = ok && write_records(f, c->nelem, [&](int64_t e, std::string& out) {
            if (size == 0) put_g(out, cell_values[e]);
            else put_mat(out, cell_values + (size_t)e * size, cell_rows, cell_cols);
            out += '\n';
        });
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) ISL_FAIL(c, ISL_ERR_ARG, std::string("write failed: ") + path);
    return ISL_OK;
    ISL_CATCH(c)
}

}  // extern "C"
