// medit.cpp -- medit (.mesh) files as FEDDLib reads them
// (feddlib/core/Mesh/MeshFileReader.cpp:16-106 sizes, MeshFileReader.hpp:80-128
// data; MeshUnstructured_def.hpp:1440-1500 one-based ids to zero-based):
//   Dimension 3            (or "Dimension" then "3" on the next line)
//   Vertices  n   then n lines  x y z flag
//   Tetrahedra n  then n lines  i j k l flag     (one-based node ids)
//   Triangles n   then n lines  i j k flag
//   Edges n       then n lines  i j flag
//   End
// Other keywords (MeshVersionFormatted, Corners, Ridges, ...) and their
// numbers are skipped.  The writer prints FP64 with 17 significant digits so
// a write / read round trip is exact.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/feddgpu.h"

namespace {

struct Medit {
    int dim = 3;
    int64_t nv = 0, nt = 0, ntri = 0, ned = 0;
    std::vector<double> xyz;
    std::vector<int32_t> vflag, tets, tflag, tris, triflag;
};

bool is_keyword(const char *t) { return std::isalpha((unsigned char)t[0]) != 0; }

// whitespace tokens of the whole file ('#' starts a comment to the end of line)
bool tokenize(const char *path, std::vector<std::string> &tok) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::string cur;
    bool comment = false;
    for (int c; (c = std::fgetc(f)) != EOF;) {
        if (comment) {
            if (c == '\n') comment = false;
            continue;
        }
        if (c == '#') {
            comment = true;
        } else if (std::isspace(c)) {
            if (!cur.empty()) tok.push_back(cur), cur.clear();
            continue;
        } else {
            cur.push_back((char)c);
            continue;
        }
        if (!cur.empty()) tok.push_back(cur), cur.clear();
    }
    if (!cur.empty()) tok.push_back(cur);
    std::fclose(f);
    return true;
}

// parses sizes and, when `data`, the entities; returns a fedd_status
fedd_status parse(const char *path, Medit &m, bool data) {
    std::vector<std::string> tok;
    if (!tokenize(path, tok)) return FEDD_ERR_ARG;
    size_t i = 0;
    auto num = [&](long long &v) {
        if (i >= tok.size()) return false;
        char *end = nullptr;
        v = std::strtoll(tok[i].c_str(), &end, 10);
        if (!end || *end) return false;
        i++;
        return true;
    };
    auto real = [&](double &v) {
        if (i >= tok.size()) return false;
        char *end = nullptr;
        v = std::strtod(tok[i].c_str(), &end);
        if (!end || *end) return false;
        i++;
        return true;
    };
    // reads `count` rows of `nid` ids (one-based when `ids`) plus a flag
    auto rows = [&](int64_t count, int nid, std::vector<int32_t> *ids, std::vector<int32_t> *flags, int64_t nv) {
        for (int64_t r = 0; r < count; r++) {
            for (int k = 0; k < nid; k++) {
                long long v;
                if (!num(v)) return false;
                if (data && ids) {
                    if (v < 1 || (nv > 0 && v > nv)) return false;
                    ids->push_back((int32_t)(v - 1));
                }
            }
            long long fl;
            if (!num(fl)) return false;
            if (data && flags) flags->push_back((int32_t)fl);
        }
        return true;
    };
    while (i < tok.size()) {
        const std::string k = tok[i++];
        long long n = 0;
        if (k == "End") break;
        if (k == "Dimension") {
            if (!num(n) || (n != 2 && n != 3)) return FEDD_ERR_MESH;
            m.dim = (int)n;
        } else if (k == "Vertices") {
            if (!num(n) || n < 0) return FEDD_ERR_MESH;
            m.nv = n;
            for (long long r = 0; r < n; r++) {
                double x[3] = {0, 0, 0};
                for (int d = 0; d < m.dim; d++)
                    if (!real(x[d])) return FEDD_ERR_MESH;
                long long fl;
                if (!num(fl)) return FEDD_ERR_MESH;
                if (data) {
                    m.xyz.insert(m.xyz.end(), x, x + 3);
                    m.vflag.push_back((int32_t)fl);
                }
            }
        } else if (k == "Tetrahedra") {
            if (!num(n) || n < 0) return FEDD_ERR_MESH;
            m.nt = n;
            if (!rows(n, 4, &m.tets, &m.tflag, m.nv)) return FEDD_ERR_MESH;
        } else if (k == "Triangles") {
            if (!num(n) || n < 0) return FEDD_ERR_MESH;
            m.ntri = n;
            if (!rows(n, 3, &m.tris, &m.triflag, m.nv)) return FEDD_ERR_MESH;
        } else if (k == "Edges") {
            if (!num(n) || n < 0) return FEDD_ERR_MESH;
            m.ned = n;
            if (!rows(n, 2, nullptr, nullptr, m.nv)) return FEDD_ERR_MESH;
        } else {
            // unknown section: skip its numbers up to the next keyword
            while (i < tok.size() && !is_keyword(tok[i].c_str())) i++;
        }
    }
    if (m.dim != 3) return FEDD_ERR_UNSUPPORTED;
    return FEDD_OK;
}

}  // namespace

extern "C" {

fedd_status fedd_medit_sizes(const char *path, int64_t *num_nodes, int64_t *num_tets, int64_t *num_tris) {
    if (!path || !num_nodes || !num_tets || !num_tris) return FEDD_ERR_ARG;
    Medit m;
    fedd_status st = parse(path, m, false);
    if (st != FEDD_OK) return st;
    *num_nodes = m.nv;
    *num_tets = m.nt;
    *num_tris = m.ntri;
    return FEDD_OK;
}

fedd_status fedd_medit_read(const char *path, double *coords, int32_t *node_flags, int32_t *tets, int32_t *tet_flags,
                            int32_t *tris, int32_t *tri_flags) {
    if (!path) return FEDD_ERR_ARG;
    Medit m;
    fedd_status st = parse(path, m, true);
    if (st != FEDD_OK) return st;
    if (coords && !m.xyz.empty()) std::memcpy(coords, m.xyz.data(), m.xyz.size() * sizeof(double));
    if (node_flags && !m.vflag.empty()) std::memcpy(node_flags, m.vflag.data(), m.vflag.size() * sizeof(int32_t));
    if (tets && !m.tets.empty()) std::memcpy(tets, m.tets.data(), m.tets.size() * sizeof(int32_t));
    if (tet_flags && !m.tflag.empty()) std::memcpy(tet_flags, m.tflag.data(), m.tflag.size() * sizeof(int32_t));
    if (tris && !m.tris.empty()) std::memcpy(tris, m.tris.data(), m.tris.size() * sizeof(int32_t));
    if (tri_flags && !m.triflag.empty()) std::memcpy(tri_flags, m.triflag.data(), m.triflag.size() * sizeof(int32_t));
    return FEDD_OK;
}

fedd_status fedd_medit_write(const char *path, int64_t num_nodes, const double *coords, const int32_t *node_flags,
                             int64_t num_tets, const int32_t *tets, const int32_t *tet_flags, int64_t num_tris,
                             const int32_t *tris, const int32_t *tri_flags) {
    if (!path || num_nodes < 0 || num_tets < 0 || num_tris < 0) return FEDD_ERR_ARG;
    if ((num_nodes && !coords) || (num_tets && !tets) || (num_tris && !tris)) return FEDD_ERR_ARG;
    FILE *f = std::fopen(path, "w");
    if (!f) return FEDD_ERR_ARG;
    std::fprintf(f, "MeshVersionFormatted 2\n\nDimension 3\n\nVertices\n%lld\n", (long long)num_nodes);
    for (int64_t v = 0; v < num_nodes; v++)
        std::fprintf(f, "%.17g %.17g %.17g %d\n", coords[3 * v], coords[3 * v + 1], coords[3 * v + 2],
                     node_flags ? node_flags[v] : 0);
    if (num_tris) {
        std::fprintf(f, "\nTriangles\n%lld\n", (long long)num_tris);
        for (int64_t t = 0; t < num_tris; t++)
            std::fprintf(f, "%d %d %d %d\n", tris[3 * t] + 1, tris[3 * t + 1] + 1, tris[3 * t + 2] + 1,
                         tri_flags ? tri_flags[t] : 0);
    }
    std::fprintf(f, "\nTetrahedra\n%lld\n", (long long)num_tets);
    for (int64_t t = 0; t < num_tets; t++)
        std::fprintf(f, "%d %d %d %d %d\n", tets[4 * t] + 1, tets[4 * t + 1] + 1, tets[4 * t + 2] + 1,
                     tets[4 * t + 3] + 1, tet_flags ? tet_flags[t] : 0);
    std::fprintf(f, "\nEnd\n");
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok ? FEDD_OK : FEDD_ERR_ARG;
}

}  // extern "C"
