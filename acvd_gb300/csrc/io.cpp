// Triangle-mesh files for the command-line drivers: the formats vtkSurface::CreateFromFile
// and vtkSurface::WriteToFile dispatch on by file name (Common/vtkSurface.cxx:1958-2136),
// read and written by this file's own parsers from the formats' published layouts.
//
//   read : .ply (ascii, binary little / big endian), .off, .obj, .stl (ascii, binary),
//          .vtk (legacy POLYDATA, ascii or binary, both POLYGONS layouts)
//   write: .ply (binary little endian, float points), .off, .obj, .stl (binary), .vtk (ascii)
//
// The extension test is the reference's: the lower-cased name contains ".vtk", ".ply", ...
// (checked in its order).  Polygons other than triangles are rejected: the clustering path
// takes triangles.  STL stores every corner separately; corners with identical coordinates
// are merged in order of first appearance, and a triangle left with a repeated corner is
// dropped.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/acvd_gpu.h"

namespace {

thread_local std::string g_io_err;

struct MeshData {
    std::vector<double> xyz;
    std::vector<int32_t> tri;
};

int io_fail(int code, const std::string& msg) {
    g_io_err = msg;
    return code;
}

std::string lower(const char* s) {
    std::string r(s);
    for (char& c : r) c = (char)std::tolower((unsigned char)c);
    return r;
}

bool read_all(const char* path, std::string& buf) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    buf = ss.str();
    return true;
}

bool host_little_endian() {
    const uint16_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

// fixed-size scalar from raw bytes in the given byte order
template <typename T>
T load_scalar(const unsigned char* p, bool little) {
    unsigned char tmp[sizeof(T)];
    if (little == host_little_endian()) std::memcpy(tmp, p, sizeof(T));
    else for (size_t i = 0; i < sizeof(T); i++) tmp[i] = p[sizeof(T) - 1 - i];
    T v;
    std::memcpy(&v, tmp, sizeof(T));
    return v;
}

template <typename T>
void store_scalar(std::string& out, T v, bool little) {
    unsigned char tmp[sizeof(T)];
    std::memcpy(tmp, &v, sizeof(T));
    if (little != host_little_endian()) std::reverse(tmp, tmp + sizeof(T));
    out.append((const char*)tmp, sizeof(T));
}

int check_faces(const MeshData& m) {
    const int64_t nv = (int64_t)m.xyz.size() / 3;
    for (int32_t v : m.tri)
        if (v < 0 || v >= nv) return io_fail(ACVD_ERR_ARG, "a face refers to a vertex that does not exist");
    return ACVD_OK;
}

int add_polygon(MeshData& m, const std::vector<int64_t>& poly) {
    if (poly.size() != 3)
        return io_fail(ACVD_ERR_UNSUPPORTED, "a polygon with " + std::to_string(poly.size()) +
                                                 " corners: only triangle meshes are read");
    for (int64_t v : poly) {
        if (v < 0 || v > INT32_MAX) return io_fail(ACVD_ERR_ARG, "vertex index out of range");
        m.tri.push_back((int32_t)v);
    }
    return ACVD_OK;
}

// ---------------------------------------------------------------- PLY
enum PlyType { kI8, kU8, kI16, kU16, kI32, kU32, kF32, kF64, kBad };

PlyType ply_type(const std::string& s) {
    if (s == "char" || s == "int8") return kI8;
    if (s == "uchar" || s == "uint8") return kU8;
    if (s == "short" || s == "int16") return kI16;
    if (s == "ushort" || s == "uint16") return kU16;
    if (s == "int" || s == "int32") return kI32;
    if (s == "uint" || s == "uint32") return kU32;
    if (s == "float" || s == "float32") return kF32;
    if (s == "double" || s == "float64") return kF64;
    return kBad;
}

int ply_size(PlyType t) {
    switch (t) {
        case kI8: case kU8: return 1;
        case kI16: case kU16: return 2;
        case kI32: case kU32: case kF32: return 4;
        case kF64: return 8;
        default: return 0;
    }
}

double ply_load(PlyType t, const unsigned char* p, bool little) {
    switch (t) {
        case kI8: return (double)(int8_t)p[0];
        case kU8: return (double)p[0];
        case kI16: return (double)load_scalar<int16_t>(p, little);
        case kU16: return (double)load_scalar<uint16_t>(p, little);
        case kI32: return (double)load_scalar<int32_t>(p, little);
        case kU32: return (double)load_scalar<uint32_t>(p, little);
        case kF32: return (double)load_scalar<float>(p, little);
        case kF64: return load_scalar<double>(p, little);
        default: return 0.0;
    }
}

struct PlyProp {
    std::string name;
    bool list = false;
    PlyType count = kBad, type = kBad;
};

struct PlyElem {
    std::string name;
    int64_t n = 0;
    std::vector<PlyProp> props;
};

int read_ply(const std::string& buf, MeshData& m) {
    size_t end = buf.find("end_header");
    if (buf.compare(0, 3, "ply") != 0 || end == std::string::npos) return io_fail(ACVD_ERR_ARG, "not a PLY file");
    size_t body = buf.find('\n', end);
    if (body == std::string::npos) return io_fail(ACVD_ERR_ARG, "PLY header without a line end");
    body++;
    std::istringstream hs(buf.substr(0, end));
    std::string line, fmt;
    std::vector<PlyElem> elems;
    while (std::getline(hs, line)) {
        std::istringstream ls(line);
        std::string kw;
        ls >> kw;
        if (kw == "format") ls >> fmt;
        else if (kw == "element") {
            PlyElem e;
            ls >> e.name >> e.n;
            elems.push_back(e);
        } else if (kw == "property") {
            if (elems.empty()) return io_fail(ACVD_ERR_ARG, "PLY property before any element");
            PlyProp p;
            std::string t;
            ls >> t;
            if (t == "list") {
                std::string c, v;
                ls >> c >> v >> p.name;
                p.list = true;
                p.count = ply_type(c);
                p.type = ply_type(v);
                if (p.count == kBad || p.type == kBad) return io_fail(ACVD_ERR_ARG, "PLY list of unknown type");
            } else {
                p.type = ply_type(t);
                ls >> p.name;
                if (p.type == kBad) return io_fail(ACVD_ERR_ARG, "PLY property of unknown type " + t);
            }
            elems.back().props.push_back(p);
        }
    }
    const bool ascii = fmt == "ascii";
    const bool little = fmt == "binary_little_endian";
    if (!ascii && !little && fmt != "binary_big_endian") return io_fail(ACVD_ERR_ARG, "PLY format " + fmt);
    const unsigned char* p = (const unsigned char*)buf.data() + body;
    const unsigned char* pend = (const unsigned char*)buf.data() + buf.size();
    std::istringstream as(ascii ? buf.substr(body) : std::string());
    auto next_value = [&](PlyType t, double& v) -> bool {
        if (ascii) return (bool)(as >> v);
        const int s = ply_size(t);
        if (pend - p < s) return false;
        v = ply_load(t, p, little);
        p += s;
        return true;
    };
    std::vector<int64_t> poly;
    for (const PlyElem& e : elems) {
        const bool is_vertex = e.name == "vertex", is_face = e.name == "face";
        int ix = -1, iy = -1, iz = -1;
        for (size_t k = 0; k < e.props.size(); k++) {
            if (e.props[k].name == "x") ix = (int)k;
            if (e.props[k].name == "y") iy = (int)k;
            if (e.props[k].name == "z") iz = (int)k;
        }
        if (is_vertex && (ix < 0 || iy < 0 || iz < 0)) return io_fail(ACVD_ERR_ARG, "PLY vertex without x y z");
        for (int64_t r = 0; r < e.n; r++) {
            double xyz[3] = {0, 0, 0};
            bool got_face = false;
            for (size_t k = 0; k < e.props.size(); k++) {
                const PlyProp& pr = e.props[k];
                double v;
                if (!pr.list) {
                    if (!next_value(pr.type, v)) return io_fail(ACVD_ERR_ARG, "PLY body ends early");
                    if ((int)k == ix) xyz[0] = v;
                    if ((int)k == iy) xyz[1] = v;
                    if ((int)k == iz) xyz[2] = v;
                    continue;
                }
                double cnt;
                if (!next_value(pr.count, cnt) || cnt < 0) return io_fail(ACVD_ERR_ARG, "PLY body ends early");
                const bool take = is_face && !got_face && (pr.name == "vertex_indices" || pr.name == "vertex_index");
                poly.clear();
                for (int64_t j = 0; j < (int64_t)cnt; j++) {
                    if (!next_value(pr.type, v)) return io_fail(ACVD_ERR_ARG, "PLY body ends early");
                    if (take) poly.push_back((int64_t)v);
                }
                if (take) {
                    got_face = true;
                    const int rc = add_polygon(m, poly);
                    if (rc) return rc;
                }
            }
            if (is_vertex) m.xyz.insert(m.xyz.end(), xyz, xyz + 3);
        }
    }
    return check_faces(m);
}

// ---------------------------------------------------------------- OFF
// strips '#' comments
bool next_data_line(std::istream& in, std::string& line) {
    while (std::getline(in, line)) {
        const size_t h = line.find('#');
        if (h != std::string::npos) line.resize(h);
        if (line.find_first_not_of(" \t\r") != std::string::npos) return true;
    }
    return false;
}

int read_off(const std::string& buf, MeshData& m) {
    std::istringstream in(buf);
    std::string line;
    if (!next_data_line(in, line) || line.find("OFF") == std::string::npos) return io_fail(ACVD_ERR_ARG, "not an OFF file");
    std::istringstream hl(line.substr(line.find("OFF") + 3));
    int64_t nv = -1, nf = -1, ne = 0;
    if (!(hl >> nv)) {
        if (!next_data_line(in, line)) return io_fail(ACVD_ERR_ARG, "OFF without counts");
        std::istringstream cl(line);
        cl >> nv >> nf >> ne;
    } else {
        hl >> nf >> ne;
    }
    if (nv < 0 || nf < 0) return io_fail(ACVD_ERR_ARG, "OFF counts");
    for (int64_t i = 0; i < nv; i++) {
        if (!next_data_line(in, line)) return io_fail(ACVD_ERR_ARG, "OFF ends in the vertices");
        std::istringstream vl(line);
        double x, y, z;
        if (!(vl >> x >> y >> z)) return io_fail(ACVD_ERR_ARG, "OFF vertex line");
        m.xyz.insert(m.xyz.end(), {x, y, z});
    }
    std::vector<int64_t> poly;
    for (int64_t f = 0; f < nf; f++) {
        if (!next_data_line(in, line)) return io_fail(ACVD_ERR_ARG, "OFF ends in the faces");
        std::istringstream fl(line);
        int64_t n;
        if (!(fl >> n)) return io_fail(ACVD_ERR_ARG, "OFF face line");
        poly.assign(n, 0);
        for (int64_t j = 0; j < n; j++)
            if (!(fl >> poly[j])) return io_fail(ACVD_ERR_ARG, "OFF face line");
        const int rc = add_polygon(m, poly);
        if (rc) return rc;
    }
    return check_faces(m);
}

// ---------------------------------------------------------------- OBJ
int read_obj(const std::string& buf, MeshData& m) {
    std::istringstream in(buf);
    std::string line;
    std::vector<int64_t> poly;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string kw;
        if (!(ls >> kw)) continue;
        if (kw == "v") {
            double x, y, z;
            if (!(ls >> x >> y >> z)) return io_fail(ACVD_ERR_ARG, "OBJ vertex line");
            m.xyz.insert(m.xyz.end(), {x, y, z});
        } else if (kw == "f") {
            poly.clear();
            std::string tok;
            const int64_t nv = (int64_t)m.xyz.size() / 3;
            while (ls >> tok) {
                const int64_t i = std::strtoll(tok.c_str(), nullptr, 10);   // "i", "i/t", "i//n", "i/t/n"
                if (i == 0) return io_fail(ACVD_ERR_ARG, "OBJ face index 0");
                poly.push_back(i > 0 ? i - 1 : nv + i);
            }
            const int rc = add_polygon(m, poly);
            if (rc) return rc;
        }
    }
    return check_faces(m);
}

// ---------------------------------------------------------------- STL
int stl_finish(const std::vector<float>& corners, MeshData& m) {
    std::map<std::tuple<float, float, float>, int32_t> ids;
    const size_t nt = corners.size() / 9;
    for (size_t t = 0; t < nt; t++) {
        int32_t c[3];
        for (int j = 0; j < 3; j++) {
            const float* q = &corners[9 * t + 3 * j];
            auto key = std::make_tuple(q[0], q[1], q[2]);
            auto it = ids.find(key);
            if (it == ids.end()) {
                const int32_t id = (int32_t)(m.xyz.size() / 3);
                ids.emplace(key, id);
                m.xyz.insert(m.xyz.end(), {(double)q[0], (double)q[1], (double)q[2]});
                c[j] = id;
            } else {
                c[j] = it->second;
            }
        }
        if (c[0] == c[1] || c[1] == c[2] || c[0] == c[2]) continue;
        m.tri.insert(m.tri.end(), c, c + 3);
    }
    return ACVD_OK;
}

int read_stl(const std::string& buf, MeshData& m) {
    std::vector<float> corners;
    if (buf.size() >= 84) {
        const uint32_t n = load_scalar<uint32_t>((const unsigned char*)buf.data() + 80, true);
        if (buf.size() == 84 + 50 * (size_t)n) {
            corners.reserve(9 * (size_t)n);
            for (uint32_t t = 0; t < n; t++) {
                const unsigned char* r = (const unsigned char*)buf.data() + 84 + 50 * (size_t)t + 12;
                for (int j = 0; j < 9; j++) corners.push_back(load_scalar<float>(r + 4 * j, true));
            }
            return stl_finish(corners, m);
        }
    }
    std::istringstream in(buf);
    std::string tok;
    if (!(in >> tok) || lower(tok.c_str()) != "solid") return io_fail(ACVD_ERR_ARG, "not an STL file");
    while (in >> tok) {
        if (lower(tok.c_str()) != "vertex") continue;
        float x, y, z;
        if (!(in >> x >> y >> z)) return io_fail(ACVD_ERR_ARG, "STL vertex line");
        corners.insert(corners.end(), {x, y, z});
    }
    if (corners.size() % 9) return io_fail(ACVD_ERR_ARG, "STL facet with other than three vertices");
    return stl_finish(corners, m);
}

// ---------------------------------------------------------------- VTK legacy
int vtk_type_size(const std::string& t) {
    const std::string s = lower(t.c_str());
    if (s == "float") return 4;
    if (s == "double") return 8;
    if (s == "int" || s == "vtktypeint32") return 4;
    if (s == "vtktypeint64" || s == "long") return 8;
    return 0;
}

int read_vtk(const std::string& buf, MeshData& m) {
    // header: version line, title line, ASCII | BINARY, DATASET POLYDATA
    size_t pos = 0;
    auto getline = [&](std::string& line) -> bool {
        if (pos >= buf.size()) return false;
        size_t e = buf.find('\n', pos);
        if (e == std::string::npos) e = buf.size();
        line = buf.substr(pos, e - pos);
        if (!line.empty() && line.back() == '\r') line.pop_back();
        pos = e + 1;
        return true;
    };
    std::string line;
    if (!getline(line) || line.find("vtk DataFile") == std::string::npos) return io_fail(ACVD_ERR_ARG, "not a VTK file");
    getline(line);   // title
    if (!getline(line)) return io_fail(ACVD_ERR_ARG, "VTK header");
    const bool binary = lower(line.c_str()).find("binary") != std::string::npos;
    // tokens of the ascii body, or positioned reads of the binary one (big endian)
    auto skip_ws = [&]() { while (pos < buf.size() && std::isspace((unsigned char)buf[pos])) pos++; };
    auto word = [&](std::string& w) -> bool {
        skip_ws();
        size_t s = pos;
        while (pos < buf.size() && !std::isspace((unsigned char)buf[pos])) pos++;
        w = buf.substr(s, pos - s);
        return !w.empty();
    };
    auto number = [&](const std::string& type, double& v) -> bool {
        if (!binary) {
            std::string w;
            if (!word(w)) return false;
            v = std::strtod(w.c_str(), nullptr);
            return true;
        }
        const int s = vtk_type_size(type);
        if (s == 0 || pos + s > buf.size()) return false;
        const unsigned char* q = (const unsigned char*)buf.data() + pos;
        const std::string t = lower(type.c_str());
        if (t == "float") v = load_scalar<float>(q, false);
        else if (t == "double") v = load_scalar<double>(q, false);
        else if (s == 4) v = load_scalar<int32_t>(q, false);
        else v = (double)load_scalar<int64_t>(q, false);
        pos += s;
        return true;
    };
    std::string w;
    bool polydata = false;
    std::vector<int64_t> offsets, conn;
    bool have_polys = false;
    while (word(w)) {
        const std::string kw = lower(w.c_str());
        if (kw == "dataset") {
            word(w);
            polydata = lower(w.c_str()) == "polydata";
            if (!polydata) return io_fail(ACVD_ERR_UNSUPPORTED, "VTK dataset " + w + ": only POLYDATA is read");
        } else if (kw == "points") {
            std::string n, type;
            word(n);
            word(type);
            const int64_t np = std::strtoll(n.c_str(), nullptr, 10);
            if (binary) { while (pos < buf.size() && buf[pos] != '\n') pos++; pos++; }
            for (int64_t i = 0; i < 3 * np; i++) {
                double v;
                if (!number(type, v)) return io_fail(ACVD_ERR_ARG, "VTK points end early");
                m.xyz.push_back(v);
            }
        } else if (kw == "polygons" || kw == "triangle_strips" || kw == "lines" || kw == "vertices") {
            std::string a, b;
            word(a);
            word(b);
            const int64_t na = std::strtoll(a.c_str(), nullptr, 10), nb = std::strtoll(b.c_str(), nullptr, 10);
            const bool polys = kw == "polygons";
            if (kw == "triangle_strips") return io_fail(ACVD_ERR_UNSUPPORTED, "VTK triangle strips");
            // the newer layout: OFFSETS / CONNECTIVITY arrays follow
            const size_t save = pos;
            std::string next;
            word(next);
            if (lower(next.c_str()) == "offsets") {
                std::string type;
                word(type);
                if (binary) { while (pos < buf.size() && buf[pos] != '\n') pos++; pos++; }
                std::vector<int64_t> off(na);
                for (int64_t i = 0; i < na; i++) {
                    double v;
                    if (!number(type, v)) return io_fail(ACVD_ERR_ARG, "VTK offsets end early");
                    off[i] = (int64_t)v;
                }
                word(next);   // CONNECTIVITY
                word(type);
                if (binary) { while (pos < buf.size() && buf[pos] != '\n') pos++; pos++; }
                std::vector<int64_t> cn(nb);
                for (int64_t i = 0; i < nb; i++) {
                    double v;
                    if (!number(type, v)) return io_fail(ACVD_ERR_ARG, "VTK connectivity ends early");
                    cn[i] = (int64_t)v;
                }
                if (polys) { offsets = off; conn = cn; have_polys = true; }
            } else {
                pos = save;
                if (binary) { while (pos < buf.size() && buf[pos] != '\n') pos++; pos++; }
                std::vector<int64_t> off{0}, cn;
                for (int64_t c = 0; c < na; c++) {
                    double v;
                    if (!number("int", v)) return io_fail(ACVD_ERR_ARG, "VTK cells end early");
                    const int64_t k = (int64_t)v;
                    for (int64_t j = 0; j < k; j++) {
                        if (!number("int", v)) return io_fail(ACVD_ERR_ARG, "VTK cells end early");
                        cn.push_back((int64_t)v);
                    }
                    off.push_back((int64_t)cn.size());
                }
                if (polys) { offsets = off; conn = cn; have_polys = true; }
            }
        } else if (kw == "point_data" || kw == "cell_data") {
            break;   // attributes are not needed
        }
    }
    if (!polydata) return io_fail(ACVD_ERR_ARG, "VTK file without DATASET POLYDATA");
    if (have_polys) {
        std::vector<int64_t> poly;
        for (size_t c = 0; c + 1 < offsets.size(); c++) {
            poly.assign(conn.begin() + offsets[c], conn.begin() + offsets[c + 1]);
            const int rc = add_polygon(m, poly);
            if (rc) return rc;
        }
    }
    return check_faces(m);
}

// ---------------------------------------------------------------- writers
void fmt_double(std::string& out, double v) {
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", v);
    out += b;
}

std::string write_ply(const double* xyz, int64_t nv, const int32_t* tri, int64_t nf) {
    std::string out = "ply\nformat binary_little_endian 1.0\nelement vertex " + std::to_string(nv) +
                      "\nproperty float x\nproperty float y\nproperty float z\nelement face " + std::to_string(nf) +
                      "\nproperty list uchar int vertex_indices\nend_header\n";
    for (int64_t i = 0; i < 3 * nv; i++) store_scalar<float>(out, (float)xyz[i], true);
    for (int64_t f = 0; f < nf; f++) {
        out.push_back((char)3);
        for (int j = 0; j < 3; j++) store_scalar<int32_t>(out, tri[3 * f + j], true);
    }
    return out;
}

std::string write_off(const double* xyz, int64_t nv, const int32_t* tri, int64_t nf) {
    std::string out = "OFF\n" + std::to_string(nv) + " " + std::to_string(nf) + " 0\n";
    for (int64_t i = 0; i < nv; i++) {
        for (int c = 0; c < 3; c++) {
            if (c) out += ' ';
            fmt_double(out, xyz[3 * i + c]);
        }
        out += '\n';
    }
    for (int64_t f = 0; f < nf; f++)
        out += "3 " + std::to_string(tri[3 * f]) + " " + std::to_string(tri[3 * f + 1]) + " " +
               std::to_string(tri[3 * f + 2]) + "\n";
    return out;
}

std::string write_obj(const double* xyz, int64_t nv, const int32_t* tri, int64_t nf) {
    std::string out;
    for (int64_t i = 0; i < nv; i++) {
        out += "v";
        for (int c = 0; c < 3; c++) {
            out += ' ';
            fmt_double(out, xyz[3 * i + c]);
        }
        out += '\n';
    }
    for (int64_t f = 0; f < nf; f++)
        out += "f " + std::to_string(tri[3 * f] + 1) + " " + std::to_string(tri[3 * f + 1] + 1) + " " +
               std::to_string(tri[3 * f + 2] + 1) + "\n";
    return out;
}

std::string write_stl(const double* xyz, int64_t nv, const int32_t* tri, int64_t nf) {
    (void)nv;
    std::string out(80, '\0');
    std::memcpy(&out[0], "binary STL", 10);
    store_scalar<uint32_t>(out, (uint32_t)nf, true);
    for (int64_t f = 0; f < nf; f++) {
        const double* a = xyz + 3 * (int64_t)tri[3 * f];
        const double* b = xyz + 3 * (int64_t)tri[3 * f + 1];
        const double* c = xyz + 3 * (int64_t)tri[3 * f + 2];
        const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const double v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
        const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 3; k++) store_scalar<float>(out, (float)(l > 0 ? n[k] / l : 0.0), true);
        for (const double* p : {a, b, c})
            for (int k = 0; k < 3; k++) store_scalar<float>(out, (float)p[k], true);
        out.append(2, '\0');
    }
    return out;
}

std::string write_vtk(const double* xyz, int64_t nv, const int32_t* tri, int64_t nf) {
    std::string out = "# vtk DataFile Version 4.2\nvtk output\nASCII\nDATASET POLYDATA\nPOINTS " +
                      std::to_string(nv) + " double\n";
    for (int64_t i = 0; i < nv; i++) {
        for (int c = 0; c < 3; c++) {
            if (c) out += ' ';
            fmt_double(out, xyz[3 * i + c]);
        }
        out += '\n';
    }
    out += "POLYGONS " + std::to_string(nf) + " " + std::to_string(4 * nf) + "\n";
    for (int64_t f = 0; f < nf; f++)
        out += "3 " + std::to_string(tri[3 * f]) + " " + std::to_string(tri[3 * f + 1]) + " " +
               std::to_string(tri[3 * f + 2]) + "\n";
    return out;
}

}  // namespace

extern "C" {

const char* acvd_io_last_error(void) { return g_io_err.c_str(); }

void acvd_free(void* p) { std::free(p); }

int acvd_read_mesh(const char* path, double** xyz, int64_t* n_vertices, int32_t** tri, int64_t* n_faces) {
    if (!path || !xyz || !n_vertices || !tri || !n_faces) return io_fail(ACVD_ERR_ARG, "null argument");
    *xyz = nullptr;
    *tri = nullptr;
    *n_vertices = *n_faces = 0;
    std::string buf;
    if (!read_all(path, buf)) return io_fail(ACVD_ERR_ARG, std::string("cannot read ") + path);
    const std::string name = lower(path);
    MeshData m;
    int rc;
    if (name.find(".vtk") != std::string::npos) rc = read_vtk(buf, m);
    else if (name.find(".vtp") != std::string::npos)
        return io_fail(ACVD_ERR_UNSUPPORTED, "VTK XML (.vtp) is not read by this build");
    else if (name.find(".ply") != std::string::npos) rc = read_ply(buf, m);
    else if (name.find(".wrl") != std::string::npos)
        return io_fail(ACVD_ERR_UNSUPPORTED, "VRML import needs a render window; not read by this build");
    else if (name.find(".off") != std::string::npos) rc = read_off(buf, m);
    else if (name.find(".obj") != std::string::npos) rc = read_obj(buf, m);
    else if (name.find(".stl") != std::string::npos) rc = read_stl(buf, m);
    else return io_fail(ACVD_ERR_UNSUPPORTED, std::string("unknown mesh file type: ") + path);
    if (rc) return rc;
    if (m.xyz.size() / 3 > (size_t)INT32_MAX) return io_fail(ACVD_ERR_UNSUPPORTED, "more than 2^31 vertices");
    *xyz = (double*)std::malloc(std::max<size_t>(m.xyz.size(), 1) * sizeof(double));
    *tri = (int32_t*)std::malloc(std::max<size_t>(m.tri.size(), 1) * sizeof(int32_t));
    if (!*xyz || !*tri) {
        std::free(*xyz);
        std::free(*tri);
        *xyz = nullptr;
        *tri = nullptr;
        return io_fail(ACVD_ERR_ARG, "out of host memory");
    }
    std::memcpy(*xyz, m.xyz.data(), m.xyz.size() * sizeof(double));
    std::memcpy(*tri, m.tri.data(), m.tri.size() * sizeof(int32_t));
    *n_vertices = (int64_t)m.xyz.size() / 3;
    *n_faces = (int64_t)m.tri.size() / 3;
    return ACVD_OK;
}

int acvd_write_mesh(const char* path, const double* xyz, int64_t n_vertices, const int32_t* tri, int64_t n_faces) {
    if (!path || (n_vertices && !xyz) || (n_faces && !tri) || n_vertices < 0 || n_faces < 0)
        return io_fail(ACVD_ERR_ARG, "null or negative argument");
    for (int64_t i = 0; i < 3 * n_faces; i++)
        if (tri[i] < 0 || tri[i] >= n_vertices) return io_fail(ACVD_ERR_ARG, "a face refers to a missing vertex");
    const std::string name = lower(path);
    std::string out;
    if (name.find(".vtk") != std::string::npos) out = write_vtk(xyz, n_vertices, tri, n_faces);
    else if (name.find(".ply") != std::string::npos) out = write_ply(xyz, n_vertices, tri, n_faces);
    else if (name.find(".stl") != std::string::npos) out = write_stl(xyz, n_vertices, tri, n_faces);
    else if (name.find(".off") != std::string::npos) out = write_off(xyz, n_vertices, tri, n_faces);
    else if (name.find(".obj") != std::string::npos) out = write_obj(xyz, n_vertices, tri, n_faces);
    else return io_fail(ACVD_ERR_UNSUPPORTED, std::string("unknown mesh file type: ") + path);
    std::ofstream f(path, std::ios::binary);
    if (!f) return io_fail(ACVD_ERR_ARG, std::string("cannot write ") + path);
    f.write(out.data(), (std::streamsize)out.size());
    return f ? ACVD_OK : io_fail(ACVD_ERR_ARG, std::string("write failed: ") + path);
}

}  // extern "C"
