// Tet-mesh input: TetGen .node/.ele/.face and Gmsh 2.x .msh (ASCII or
// binary), the per-body placement transform, boundary-triangle extraction
// and surface edges.  Host code; its output feeds pdgb_create /
// pdgb_create_batch.
//
// Behaviour follows the reference's DataLoader (src/simulation/
// dataLoader.cu:38-290) and its Gmsh reader (src/simulation/MshLoader.cpp):
//   - .node: first line holds the vertex count; each following line
//     "id x y z ..." gives the next vertex (the id is not used); optional
//     centring subtracts the float centroid and swaps y and z
//     (dataLoader.cu:131-171);
//   - .ele / .face: first line holds the count; lines "id a b c [d] ..." give
//     corner ids minus the body's start index (dataLoader.cu:38-90);
//   - without a .face file (or with an empty one) the surface is the set of
//     tet faces that occur once, faces taken as (0,1,2), (0,2,3), (0,3,1),
//     (1,3,2) of each tet, listed in ascending order of their sorted corner
//     triples (dataLoader.cu:91-126);
//   - edges: the distinct triangle edges, ascending (dataLoader.cu:173-200);
//   - placement: X <- translate(pos) scale(s) rotX rotY rotZ X, angles in
//     degrees, evaluated in float (dataLoader.cu:209-217, TransformVertices
//     utilities.cu:57-65).
// Extensions: '#' comment and blank lines are skipped; a start index of -1
// takes the first .node id as the base; a .msh body keeps only its
// tetrahedra (type 4, and the corner nodes of type 11), where the reference
// divides the node list of all elements by 4.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "engine.h"

namespace pdgb {
namespace {

std::string read_file(const char* path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error{PDGB_ERR_NOT_FOUND, std::string("cannot open ") + path};
    return std::string(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

// Lines of a TetGen file without comments and blank lines.
struct LineReader {
    const std::string& s;
    size_t pos = 0;
    explicit LineReader(const std::string& str) : s(str) {}
    bool next(std::string& line) {
        while (pos < s.size()) {
            size_t e = s.find('\n', pos);
            if (e == std::string::npos) e = s.size();
            line.assign(s, pos, e - pos);
            pos = e + 1;
            const size_t h = line.find('#');
            if (h != std::string::npos) line.resize(h);
            if (line.find_first_not_of(" \t\r") != std::string::npos) return true;
        }
        return false;
    }
};

long long parse_count(LineReader& r, const char* what, const char* path) {
    std::string line;
    if (!r.next(line)) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": missing " + what + " count"};
    char* end = nullptr;
    errno = 0;
    const long long n = std::strtoll(line.c_str(), &end, 10);
    if (end == line.c_str() || errno || n < 0 || n > (1LL << 28))
        throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": bad " + what + " count"};
    return n;
}

// Parses up to k integers (after the leading id) of one record line.
int parse_ids(const std::string& line, long long* out, int k) {
    const char* p = line.c_str();
    char* end = nullptr;
    std::strtoll(p, &end, 10);  // record id
    if (end == p) return -1;
    p = end;
    int got = 0;
    for (; got < k; ++got) {
        errno = 0;
        const long long v = std::strtoll(p, &end, 10);
        if (end == p || errno) break;
        out[got] = v;
        p = end;
    }
    return got;
}

std::vector<float> load_node(const char* path, int* first_id) {
    const std::string txt = read_file(path);
    LineReader r(txt);
    const long long n = parse_count(r, "vertex", path);
    std::vector<float> X(3 * (size_t)n);
    std::string line;
    for (long long i = 0; i < n; ++i) {
        if (!r.next(line)) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": fewer vertices than declared"};
        const char* p = line.c_str();
        char* end = nullptr;
        const long long id = std::strtoll(p, &end, 10);
        if (end == p) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": bad vertex line"};
        if (i == 0 && first_id) *first_id = (int)id;
        p = end;
        for (int d = 0; d < 3; ++d) {
            const float v = std::strtof(p, &end);
            if (end == p) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": bad vertex coordinate"};
            X[3 * (size_t)i + d] = v;
            p = end;
        }
    }
    return X;
}

std::vector<uint32_t> load_records(const char* path, int per, long long nv, int start, const char* what) {
    const std::string txt = read_file(path);
    LineReader r(txt);
    const long long n = parse_count(r, what, path);
    std::vector<uint32_t> out((size_t)n * per);
    std::string line;
    long long ids[8];
    for (long long i = 0; i < n; ++i) {
        if (!r.next(line)) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": fewer " + what + "s than declared"};
        if (parse_ids(line, ids, per) != per) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": bad " + what};
        for (int k = 0; k < per; ++k) {
            const long long v = ids[k] - start;
            if (v < 0 || v >= nv)
                throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": " + what + " corner out of range"};
            out[(size_t)i * per + k] = (uint32_t)v;
        }
    }
    return out;
}

// ---- Gmsh 2.x
template <class T> T take(const std::string& s, size_t& pos) {
    if (pos + sizeof(T) > s.size()) throw Error{PDGB_ERR_BAD_MESH, "msh: truncated binary section"};
    T v;
    std::memcpy(&v, s.data() + pos, sizeof(T));
    pos += sizeof(T);
    return v;
}

int nodes_of_type(int t) {
    switch (t) {
        case 1: return 2;   case 2: return 3;   case 3: return 4;   case 4: return 4;
        case 5: return 8;   case 6: return 6;   case 7: return 5;   case 8: return 3;
        case 9: return 6;   case 10: return 9;  case 11: return 10; case 12: return 27;
        case 13: return 18; case 14: return 14; case 15: return 1;  case 16: return 8;
        case 17: return 20; case 18: return 15; case 19: return 13;
        default: return -1;
    }
}

void load_msh(const char* path, std::vector<float>& X, std::vector<uint32_t>& tets) {
    const std::string s = read_file(path);
    std::istringstream in(s);
    std::string tok;
    in >> tok;
    if (tok != "$MeshFormat") throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": not a Gmsh file"};
    double version = 0;
    int type = 0, dsize = 0;
    in >> version >> type >> dsize;
    if (!(version >= 2.0 && version <= 2.2)) throw Error{PDGB_ERR_UNSUPPORTED, std::string(path) + ": Gmsh version"};
    const bool binary = type == 1;
    if (dsize != 8) throw Error{PDGB_ERR_UNSUPPORTED, std::string(path) + ": data size must be 8"};
    size_t pos = (size_t)in.tellg();
    auto skip_ws = [&] {
        while (pos < s.size() && (s[pos] == ' ' || s[pos] == '\n' || s[pos] == '\r' || s[pos] == '\t')) ++pos;
    };
    // binary blocks start right after the newline that ends the count line
    // (whitespace skipping could eat data bytes such as 0x0A)
    auto skip_newline = [&] {
        if (pos < s.size() && s[pos] == '\r') ++pos;
        if (pos < s.size() && s[pos] == '\n') ++pos;
    };
    if (binary) {
        skip_ws();
        if (take<int32_t>(s, pos) != 1) throw Error{PDGB_ERR_UNSUPPORTED, std::string(path) + ": endianness"};
    }
    auto word = [&]() {
        skip_ws();
        size_t e = pos;
        while (e < s.size() && !std::isspace((unsigned char)s[e])) ++e;
        std::string w = s.substr(pos, e - pos);
        pos = e;
        return w;
    };
    auto number = [&]() -> long long {
        const std::string w = word();
        char* end = nullptr;
        const long long v = std::strtoll(w.c_str(), &end, 10);
        if (w.empty() || *end) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": bad number"};
        return v;
    };
    auto real = [&]() -> double {
        const std::string w = word();
        char* end = nullptr;
        const double v = std::strtod(w.c_str(), &end);
        if (w.empty() || *end) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": bad coordinate"};
        return v;
    };
    if (word() != "$EndMeshFormat") throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": bad header"};
    std::vector<double> nodes;
    bool have_nodes = false;
    while (true) {
        const std::string sec = word();
        if (sec.empty()) break;
        if (sec == "$Nodes") {
            const long long n = number();
            if (n < 0 || n > (1LL << 28)) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": node count"};
            nodes.assign(3 * (size_t)n, 0.0);
            if (binary) skip_newline();
            for (long long i = 0; i < n; ++i) {
                const long long id = binary ? take<int32_t>(s, pos) : number();
                if (id < 1 || id > n) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": node ids must be 1..n"};
                for (int d = 0; d < 3; ++d) nodes[3 * (size_t)(id - 1) + d] = binary ? take<double>(s, pos) : real();
            }
            have_nodes = true;
            if (word() != "$EndNodes") throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": $EndNodes"};
        } else if (sec == "$Elements") {
            const long long n = number();
            if (n < 0 || n > (1LL << 30)) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": element count"};
            auto add = [&](int etype, const std::vector<long long>& nd) {
                if (etype != 4 && etype != 11) return;
                for (int k = 0; k < 4; ++k) {
                    if (nd[k] < 1) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": element node id"};
                    tets.push_back((uint32_t)(nd[k] - 1));
                }
            };
            std::vector<long long> nd;
            if (binary) {
                skip_newline();
                long long done = 0;
                while (done < n) {
                    const int etype = take<int32_t>(s, pos);
                    const int count = take<int32_t>(s, pos);
                    const int ntags = take<int32_t>(s, pos);
                    const int nn = nodes_of_type(etype);
                    if (nn < 0 || count < 0 || ntags < 0) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": element type"};
                    for (int e = 0; e < count; ++e) {
                        take<int32_t>(s, pos);  // element id
                        for (int t = 0; t < ntags; ++t) take<int32_t>(s, pos);
                        nd.resize(nn);
                        for (int k = 0; k < nn; ++k) nd[k] = take<int32_t>(s, pos);
                        add(etype, nd);
                    }
                    done += count;
                }
            } else {
                for (long long e = 0; e < n; ++e) {
                    number();  // element id
                    const int etype = (int)number();
                    const int ntags = (int)number();
                    for (int t = 0; t < ntags; ++t) number();
                    const int nn = nodes_of_type(etype);
                    if (nn < 0) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": element type"};
                    nd.resize(nn);
                    for (int k = 0; k < nn; ++k) nd[k] = number();
                    add(etype, nd);
                }
            }
            if (word() != "$EndElements") throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": $EndElements"};
        } else if (sec[0] == '$') {
            // unknown or data section: skip to its end tag
            const std::string endtag = "$End" + sec.substr(1);
            const size_t e = s.find(endtag, pos);
            if (e == std::string::npos) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": unterminated " + sec};
            pos = e + endtag.size();
        } else {
            throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": unexpected '" + sec + "'"};
        }
    }
    if (!have_nodes) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": no $Nodes"};
    const size_t nv = nodes.size() / 3;
    for (uint32_t t : tets)
        if (t >= nv) throw Error{PDGB_ERR_BAD_MESH, std::string(path) + ": element node out of range"};
    X.resize(nodes.size());
    for (size_t i = 0; i < nodes.size(); ++i) X[i] = (float)nodes[i];
}

// ---- placement
// Column-major 4x4 (m[c][r]), products evaluated like glm's in float.
struct M4 {
    float m[4][4];
};

M4 mul(const M4& a, const M4& b) {  // a * b
    M4 r{};
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) {
            float acc = a.m[0][k] * b.m[c][0];
            acc = acc + a.m[1][k] * b.m[c][1];
            acc = acc + a.m[2][k] * b.m[c][2];
            acc = acc + a.m[3][k] * b.m[c][3];
            r.m[c][k] = acc;
        }
    return r;
}

M4 identity() {
    M4 r{};
    for (int i = 0; i < 4; ++i) r.m[i][i] = 1.f;
    return r;
}

// Rotation by `deg` degrees about a coordinate axis (0 = x, 1 = y, 2 = z).
M4 axis_rotation(float deg, int axis) {
    const float a = deg * 0.01745329251994329576923690768489f;
    const float c = std::cos(a), s = std::sin(a);
    M4 r = identity();
    r.m[axis][axis] = c + (1.f - c);  // the axis entry as the Rodrigues form rounds it
    const int i = (axis + 1) % 3, j = (axis + 2) % 3;  // the rotated plane
    r.m[i][i] = c;
    r.m[i][j] = s;
    r.m[j][i] = -s;
    r.m[j][j] = c;
    return r;
}

void place(std::vector<float>& X, const float pos[3], const float scale[3], const float rot[3]) {
    M4 T = identity();
    for (int d = 0; d < 3; ++d) T.m[3][d] = pos[d];
    M4 S = identity();
    for (int d = 0; d < 3; ++d) S.m[d][d] = scale[d];
    M4 M = mul(mul(mul(mul(T, S), axis_rotation(rot[0], 0)), axis_rotation(rot[1], 1)), axis_rotation(rot[2], 2));
    const size_t n = X.size() / 3;
    for (size_t v = 0; v < n; ++v) {
        const float x = X[3 * v], y = X[3 * v + 1], z = X[3 * v + 2];
        for (int r = 0; r < 3; ++r) {
            float acc = M.m[0][r] * x;
            acc = acc + M.m[1][r] * y;
            acc = acc + M.m[2][r] * z;
            acc = acc + M.m[3][r];
            X[3 * v + r] = acc;
        }
    }
}

void centralize(std::vector<float>& X) {
    const size_t n = X.size() / 3;
    if (n == 0) return;
    float c[3] = {0.f, 0.f, 0.f};
    for (size_t v = 0; v < n; ++v)
        for (int d = 0; d < 3; ++d) c[d] += X[3 * v + d];
    for (int d = 0; d < 3; ++d) c[d] /= (float)n;
    for (size_t v = 0; v < n; ++v) {
        for (int d = 0; d < 3; ++d) X[3 * v + d] -= c[d];
        std::swap(X[3 * v + 1], X[3 * v + 2]);
    }
}

}  // namespace

std::vector<uint32_t> boundary_triangles(size_t nt, const uint32_t* tets) {
    using Tri = std::tuple<uint32_t, uint32_t, uint32_t>;
    static const int kFace[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
    std::map<Tri, Tri> oriented;  // sorted key -> face as the tet lists it
    std::set<Tri> once;
    for (size_t t = 0; t < nt; ++t) {
        const uint32_t* q = tets + 4 * t;
        for (const auto& f : kFace) {
            uint32_t a = q[f[0]], b = q[f[1]], c = q[f[2]];
            const Tri face{a, b, c};
            if (a > b) std::swap(a, b);
            if (b > c) std::swap(b, c);
            if (a > b) std::swap(a, b);
            const Tri key{a, b, c};
            oriented[key] = face;
            auto it = once.find(key);
            if (it == once.end()) once.insert(key);
            else once.erase(it);
        }
    }
    std::vector<uint32_t> out;
    out.reserve(3 * once.size());
    for (const Tri& k : once) {
        const Tri& f = oriented[k];
        out.push_back(std::get<0>(f));
        out.push_back(std::get<1>(f));
        out.push_back(std::get<2>(f));
    }
    return out;
}

std::vector<uint32_t> surface_edges(const std::vector<uint32_t>& tris) {
    std::set<std::pair<uint32_t, uint32_t>> e;
    for (size_t i = 0; i + 2 < tris.size(); i += 3)
        for (int k = 0; k < 3; ++k) e.insert(std::minmax(tris[i + k], tris[i + (k + 1) % 3]));
    std::vector<uint32_t> out;
    out.reserve(2 * e.size());
    for (const auto& p : e) {
        out.push_back(p.first);
        out.push_back(p.second);
    }
    return out;
}

void load_body_file(const pdgb_body_file& f, std::vector<float>& X, std::vector<uint32_t>& tets,
                    std::vector<uint32_t>& tris) {
    const bool tetgen = f.node_file && *f.node_file;
    if (tetgen) {
        if (!f.ele_file || !*f.ele_file) throw Error{PDGB_ERR_INVALID_ARGUMENT, "a .node file needs an .ele file"};
        int first = 0;
        X = load_node(f.node_file, &first);
        const int start = f.start_index == -1 ? first : f.start_index;
        const long long nv = (long long)(X.size() / 3);
        tets = load_records(f.ele_file, 4, nv, start, "tet");
        if (f.face_file && *f.face_file) {
            std::ifstream probe(f.face_file);
            if (probe) tris = load_records(f.face_file, 3, nv, start, "face");  // a missing .face is optional
        }
        if (f.centralize) centralize(X);
        if (tris.empty()) tris = boundary_triangles(tets.size() / 4, tets.data());
    } else if (f.msh_file && *f.msh_file) {
        load_msh(f.msh_file, X, tets);  // no centring and no surface for .msh bodies (dataLoader.cu:235-270)
    } else {
        throw Error{PDGB_ERR_INVALID_ARGUMENT, "no .node or .msh file given"};
    }
    if (tets.empty()) throw Error{PDGB_ERR_BAD_MESH, "the file holds no tetrahedra"};
    place(X, f.pos, f.scale, f.rot);
}

}  // namespace pdgb

using namespace pdgb;

namespace {
template <class T> T* dup(const std::vector<T>& v) {
    T* p = (T*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(T));
    if (!p) throw std::bad_alloc();
    if (!v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}
}  // namespace

extern "C" {

int pdgb_load_body_file(const pdgb_body_file* f, pdgb_tet_mesh** out) {
    if (!f || !out) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "file descriptor or out is null");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    try {
        std::vector<float> X;
        std::vector<uint32_t> tets, tris;
        load_body_file(*f, X, tets, tris);
        const std::vector<uint32_t> edges = surface_edges(tris);
        pdgb_tet_mesh* m = (pdgb_tet_mesh*)std::calloc(1, sizeof(pdgb_tet_mesh));
        if (!m) throw std::bad_alloc();
        m->num_verts = (int)(X.size() / 3);
        m->num_tets = (int)(tets.size() / 4);
        m->num_tris = (int)(tris.size() / 3);
        m->num_edges = (int)(edges.size() / 2);
        m->X = dup(X);
        m->tets = dup(tets);
        m->tris = dup(tris);
        m->edges = dup(edges);
        *out = m;
        return PDGB_OK;
    } catch (const Error& e) {
        set_last_error(e.status, e.msg);
        return e.status;
    } catch (const std::bad_alloc&) {
        set_last_error(PDGB_ERR_OUT_OF_MEMORY, "host allocation failed");
        return PDGB_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        set_last_error(PDGB_ERR_BAD_MESH, e.what());
        return PDGB_ERR_BAD_MESH;
    }
}

void pdgb_free_tet_mesh(pdgb_tet_mesh* m) {
    if (!m) return;
    std::free(m->X);
    std::free(m->tets);
    std::free(m->tris);
    std::free(m->edges);
    std::free(m);
}

int pdgb_surface_triangles(int num_tets, const uint32_t* tets, uint32_t* tris, long long capacity, int* num_tris) {
    if (num_tets < 0 || (num_tets > 0 && !tets) || !num_tris || capacity < 0 || (capacity > 0 && !tris)) {
        set_last_error(PDGB_ERR_INVALID_ARGUMENT, "bad arguments");
        return PDGB_ERR_INVALID_ARGUMENT;
    }
    try {
        const std::vector<uint32_t> t = boundary_triangles((size_t)num_tets, tets);
        *num_tris = (int)(t.size() / 3);
        if ((long long)t.size() > 3 * capacity) {
            set_last_error(PDGB_ERR_INVALID_ARGUMENT, "capacity too small");
            return PDGB_ERR_INVALID_ARGUMENT;
        }
        if (!t.empty()) std::memcpy(tris, t.data(), t.size() * sizeof(uint32_t));
        return PDGB_OK;
    } catch (const std::bad_alloc&) {
        set_last_error(PDGB_ERR_OUT_OF_MEMORY, "host allocation failed");
        return PDGB_ERR_OUT_OF_MEMORY;
    }
}

}  // extern "C"
