// Triangle-mesh files for the command-line drivers: the formats vtkSurface::CreateFromFile
// and vtkSurface::WriteToFile dispatch on by file name (Common/vtkSurface.cxx:1958-2136),
// read and written by this file's own parsers from the formats' published layouts.
//
//   read : .ply (ascii, binary little / big endian), .off, .obj, .stl (ascii, binary),
//          .vtk (legacy POLYDATA, ascii or binary, both POLYGONS layouts),
//          .vtp (VTK XML PolyData: ascii, base64 or appended data, zlib-compressed or not)
//   write: .ply (binary little endian, float points), .off, .obj, .stl (binary), .vtk (ascii),
//          .vtp (inline base64, uncompressed)
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

// ---------------------------------------------------------------- zlib inflate
// Decoder for zlib streams (RFC 1950) holding DEFLATE data (RFC 1951), written from the
// two specifications: stored, fixed-Huffman and dynamic-Huffman blocks; canonical
// Huffman codes (RFC 1951 sec. 3.2.2) decoded one bit at a time from the per-length
// code counts; the Adler-32 checksum verified.  VTK's XML writers compress their data
// arrays with it by default.
class BitReader {
public:
    BitReader(const unsigned char* p, size_t n) : p_(p), n_(n) {}
    // `count` bits, least significant first (count <= 16)
    uint32_t take(int count) {
        while (have_ < count) {
            if (pos_ >= n_) {
                failed_ = true;
                return 0;
            }
            acc_ |= (uint32_t)p_[pos_++] << have_;
            have_ += 8;
        }
        const uint32_t v = acc_ & ((1u << count) - 1u);
        acc_ >>= count;
        have_ -= count;
        return v;
    }
    void to_byte() {   // drop the bits left in the current byte
        acc_ = 0;
        have_ = 0;
    }
    size_t pos() const { return pos_; }
    bool failed() const { return failed_; }
    const unsigned char* data() const { return p_; }
    size_t size() const { return n_; }
    void skip(size_t bytes) { pos_ += bytes; }

private:
    const unsigned char* p_;
    size_t n_, pos_ = 0;
    uint32_t acc_ = 0;
    int have_ = 0;
    bool failed_ = false;
};

// canonical code: symbols sorted by (code length, symbol); the codes of one length are
// consecutive integers starting at first_code[len]
struct Canonical {
    int count[16] = {0};
    int first_code[16] = {0};
    int first_index[16] = {0};
    std::vector<int> sorted;
    bool build(const uint8_t* len, int n) {
        for (int l = 0; l < 16; l++) count[l] = 0;
        for (int s = 0; s < n; s++) count[len[s]]++;
        count[0] = 0;
        int code = 0, index = 0;
        for (int l = 1; l < 16; l++) {
            code = (code + (l > 1 ? count[l - 1] : 0)) << (l > 1 ? 1 : 0);
            first_code[l] = code;
            first_index[l] = index;
            index += count[l];
            if (count[l] > (1 << l)) return false;
        }
        // over-subscription: more codes than the lengths can hold
        long room = 1;
        for (int l = 1; l < 16; l++) {
            room = 2 * room - count[l];
            if (room < 0) return false;
        }
        sorted.assign(index, 0);
        std::vector<int> next(16);
        for (int l = 1; l < 16; l++) next[l] = first_index[l];
        for (int s = 0; s < n; s++)
            if (len[s]) sorted[next[len[s]]++] = s;
        return true;
    }
    int decode(BitReader& in) const {
        int code = 0;
        for (int l = 1; l < 16; l++) {
            code = (code << 1) | (int)in.take(1);
            if (in.failed()) return -1;
            const int d = code - first_code[l];
            if (d >= 0 && d < count[l]) return sorted[first_index[l] + d];
        }
        return -1;
    }
};

bool inflate_deflate(BitReader& in, std::string& out, size_t limit) {
    // length and distance bases of RFC 1951 sec. 3.2.5, built from their pattern
    int len_base[29], len_extra[29], dist_base[30], dist_extra[30];
    for (int i = 0; i < 8; i++) { len_base[i] = 3 + i; len_extra[i] = 0; }
    for (int i = 8, base = 11; i < 28; i++) {
        len_extra[i] = (i - 4) / 4;
        len_base[i] = base;
        base += 1 << len_extra[i];
    }
    len_base[28] = 258;
    len_extra[28] = 0;
    for (int i = 0; i < 4; i++) { dist_base[i] = 1 + i; dist_extra[i] = 0; }
    for (int i = 4, base = 5; i < 30; i++) {
        dist_extra[i] = (i - 2) / 2;
        dist_base[i] = base;
        base += 1 << dist_extra[i];
    }
    static const int kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    for (;;) {
        const uint32_t final_block = in.take(1);
        const uint32_t type = in.take(2);
        if (in.failed()) return false;
        if (type == 0) {   // stored
            in.to_byte();
            const size_t at = in.pos();
            if (at + 4 > in.size()) return false;
            const unsigned char* q = in.data() + at;
            const unsigned len = q[0] | (q[1] << 8), nlen = q[2] | (q[3] << 8);
            if ((len ^ 0xffffu) != nlen || at + 4 + len > in.size() || out.size() + len > limit) return false;
            out.append((const char*)q + 4, len);
            in.skip(4 + len);
        } else if (type == 1 || type == 2) {
            Canonical lit, dist;
            uint8_t lens[320];
            if (type == 1) {   // fixed codes (sec. 3.2.6)
                for (int s = 0; s < 288; s++) lens[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
                for (int s = 0; s < 30; s++) lens[288 + s] = 5;
                if (!lit.build(lens, 288) || !dist.build(lens + 288, 30)) return false;
            } else {           // dynamic codes (sec. 3.2.7)
                const int nlit = (int)in.take(5) + 257, ndist = (int)in.take(5) + 1, nclen = (int)in.take(4) + 4;
                if (in.failed() || nlit > 286 || ndist > 30) return false;
                uint8_t cl[19] = {0};
                for (int i = 0; i < nclen; i++) cl[kOrder[i]] = (uint8_t)in.take(3);
                Canonical clc;
                if (!clc.build(cl, 19)) return false;
                int got = 0;
                while (got < nlit + ndist) {
                    const int sym = clc.decode(in);
                    if (sym < 0) return false;
                    if (sym < 16) {
                        lens[got++] = (uint8_t)sym;
                        continue;
                    }
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (got == 0) return false;
                        val = lens[got - 1];
                        rep = 3 + (int)in.take(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)in.take(3);
                    } else {
                        rep = 11 + (int)in.take(7);
                    }
                    if (in.failed() || got + rep > nlit + ndist) return false;
                    while (rep--) lens[got++] = val;
                }
                if (lens[256] == 0) return false;   // no end-of-block code
                if (!lit.build(lens, nlit) || !dist.build(lens + nlit, ndist)) return false;
            }
            for (;;) {
                const int sym = lit.decode(in);
                if (sym < 0) return false;
                if (sym < 256) {
                    if (out.size() >= limit) return false;
                    out.push_back((char)sym);
                    continue;
                }
                if (sym == 256) break;
                if (sym > 285) return false;
                const int length = len_base[sym - 257] + (int)in.take(len_extra[sym - 257]);
                const int dsym = dist.decode(in);
                if (dsym < 0 || dsym > 29) return false;
                const size_t d = (size_t)dist_base[dsym] + in.take(dist_extra[dsym]);
                if (in.failed() || d > out.size() || out.size() + length > limit) return false;
                const size_t from = out.size() - d;
                for (int j = 0; j < length; j++) out.push_back(out[from + j]);
            }
        } else {
            return false;
        }
        if (final_block) return true;
    }
}

uint32_t adler32(const std::string& s) {
    uint32_t a = 1, b = 0;
    for (unsigned char c : s) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

// one zlib stream (header, DEFLATE data, Adler-32) holding exactly `expect` bytes
bool zlib_inflate(const unsigned char* p, size_t n, size_t expect, std::string& out) {
    out.clear();
    if (n < 6) return false;
    const unsigned cmf = p[0], flg = p[1];
    if ((cmf & 15u) != 8u || (cmf >> 4) > 7u || ((cmf << 8) | flg) % 31u != 0u || (flg & 32u)) return false;
    BitReader in(p + 2, n - 2);
    if (!inflate_deflate(in, out, expect)) return false;
    const size_t at = 2 + in.pos();
    if (at + 4 > n || out.size() != expect) return false;
    const uint32_t want = ((uint32_t)p[at] << 24) | ((uint32_t)p[at + 1] << 16) | ((uint32_t)p[at + 2] << 8) | p[at + 3];
    return want == adler32(out);
}

// ---------------------------------------------------------------- VTK XML PolyData
// The .vtp layout of VTK's XML file formats: a VTKFile element (byte_order, header_type
// UInt32 / UInt64, optional vtkZLibDataCompressor) holding PolyData Pieces, each with a
// Points DataArray and the Polys' "connectivity" / "offsets" arrays, in ascii, inline
// base64 ("binary") or appended (raw or base64) form.  A binary block is a header -- the
// byte count, or for compressed data [blocks, block size, last block size, compressed
// sizes...] -- followed by the data.  Pieces are concatenated.  Only triangles are read;
// triangle strips are refused, vertices and lines (no faces) are ignored.
struct XmlTag {
    std::string name;
    std::map<std::string, std::string> attr;
    size_t open = 0, close = 0;   // '<' and one past '>'
    bool empty = false;           // <... />
};

// the next element tag at or after `from` (comments and declarations skipped)
bool next_tag(const std::string& s, size_t from, size_t stop, XmlTag& t) {
    size_t i = from;
    for (;;) {
        i = s.find('<', i);
        if (i == std::string::npos || i >= stop) return false;
        if (s.compare(i, 4, "<!--") == 0) {
            i = s.find("-->", i);
            if (i == std::string::npos) return false;
            continue;
        }
        if (i + 1 < s.size() && (s[i + 1] == '?' || s[i + 1] == '!' || s[i + 1] == '/')) {
            i++;
            continue;
        }
        break;
    }
    const size_t end = s.find('>', i);
    if (end == std::string::npos) return false;
    t = XmlTag();
    t.open = i;
    t.close = end + 1;
    t.empty = s[end - 1] == '/';
    size_t k = i + 1;
    while (k < end && !std::isspace((unsigned char)s[k]) && s[k] != '/' && s[k] != '>') t.name += s[k++];
    for (;;) {
        while (k < end && (std::isspace((unsigned char)s[k]) || s[k] == '/')) k++;
        if (k >= end) break;
        std::string key;
        while (k < end && s[k] != '=' && !std::isspace((unsigned char)s[k])) key += s[k++];
        while (k < end && s[k] != '"' && s[k] != '\'') k++;
        if (k >= end) break;
        const char q = s[k++];
        const size_t v = k;
        while (k < end && s[k] != q) k++;
        t.attr[key] = s.substr(v, k - v);
        k++;
    }
    return true;
}

std::string attr_of(const XmlTag& t, const char* key, const char* dflt = "") {
    const auto it = t.attr.find(key);
    return it == t.attr.end() ? std::string(dflt) : it->second;
}

int b64_value(unsigned char c) {
    if (c >= 'A' && c <= 'Z') return c - 'A';
    if (c >= 'a' && c <= 'z') return c - 'a' + 26;
    if (c >= '0' && c <= '9') return c - '0' + 52;
    if (c == '+') return 62;
    if (c == '/') return 63;
    return -1;
}

// base64 text to bytes; '=' ends a quantum, after which decoding starts afresh, so text
// made of separately encoded pieces (VTK encodes a compressed block's header apart from
// its data) decodes to the pieces' concatenation
bool b64_decode(const char* p, size_t n, std::string& out) {
    out.clear();
    uint32_t acc = 0;
    int have = 0;
    for (size_t i = 0; i < n; i++) {
        const unsigned char c = (unsigned char)p[i];
        if (std::isspace(c)) continue;
        if (c == '=') {
            acc = 0;
            have = 0;
            continue;
        }
        const int v = b64_value(c);
        if (v < 0) return false;
        acc = (acc << 6) | (uint32_t)v;
        have += 6;
        if (have >= 8) {
            have -= 8;
            out.push_back((char)((acc >> have) & 0xffu));
        }
    }
    return true;
}

void b64_encode(const std::string& in, std::string& out) {
    static const char* kAlphabet = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    size_t i = 0;
    for (; i + 3 <= in.size(); i += 3) {
        const uint32_t v = ((uint32_t)(unsigned char)in[i] << 16) | ((uint32_t)(unsigned char)in[i + 1] << 8) |
                           (unsigned char)in[i + 2];
        for (int s = 18; s >= 0; s -= 6) out += kAlphabet[(v >> s) & 63u];
    }
    const size_t rest = in.size() - i;
    if (rest) {
        uint32_t v = (uint32_t)(unsigned char)in[i] << 16;
        if (rest == 2) v |= (uint32_t)(unsigned char)in[i + 1] << 8;
        out += kAlphabet[(v >> 18) & 63u];
        out += kAlphabet[(v >> 12) & 63u];
        out += rest == 2 ? kAlphabet[(v >> 6) & 63u] : '=';
        out += '=';
    }
}

struct VtpFile {
    bool little = true;
    int header_bytes = 4;         // UInt32 / UInt64
    bool zlib = false;
    std::string appended;         // the appended data after '_' (raw), or its base64 text
    bool appended_b64 = false;
    std::vector<size_t> offsets;  // every appended DataArray offset, sorted (base64 piece ends)
};

uint64_t vtp_header_value(const VtpFile& f, const unsigned char* p) {
    return f.header_bytes == 8 ? load_scalar<uint64_t>(p, f.little) : load_scalar<uint32_t>(p, f.little);
}

// a binary block (header + data) to the array's raw bytes; `avail` bounds the block
bool vtp_block(const VtpFile& f, const unsigned char* p, size_t avail, std::string& raw) {
    const size_t hb = (size_t)f.header_bytes;
    if (!f.zlib) {
        if (avail < hb) return false;
        const uint64_t nbytes = vtp_header_value(f, p);
        if (nbytes > avail - hb) return false;
        raw.assign((const char*)p + hb, (size_t)nbytes);
        return true;
    }
    if (avail < 3 * hb) return false;
    const uint64_t nblocks = vtp_header_value(f, p), bsize = vtp_header_value(f, p + hb),
                   last = vtp_header_value(f, p + 2 * hb);
    if (nblocks > (avail - 3 * hb) / hb) return false;
    size_t at = (3 + (size_t)nblocks) * hb;
    raw.clear();
    std::string part;
    for (uint64_t b = 0; b < nblocks; b++) {
        const uint64_t csize = vtp_header_value(f, p + (3 + b) * hb);
        const uint64_t usize = (b + 1 == nblocks && last != 0) ? last : bsize;
        if (csize > avail - at || usize > ((uint64_t)1 << 40)) return false;
        if (!zlib_inflate(p + at, (size_t)csize, (size_t)usize, part)) return false;
        raw += part;
        at += (size_t)csize;
    }
    return true;
}

bool vtp_type(const std::string& t, int& size, bool& is_float, bool& is_signed) {
    is_float = t == "Float32" || t == "Float64";
    is_signed = t[0] == 'I' || is_float;
    if (t == "Int8" || t == "UInt8") size = 1;
    else if (t == "Int16" || t == "UInt16") size = 2;
    else if (t == "Int32" || t == "UInt32" || t == "Float32") size = 4;
    else if (t == "Int64" || t == "UInt64" || t == "Float64") size = 8;
    else return false;
    return true;
}

// one DataArray's values, as doubles (coordinates) or integers (ids)
int vtp_array(const std::string& s, const VtpFile& f, const XmlTag& t, std::vector<double>* dv,
              std::vector<int64_t>* iv) {
    const std::string type = attr_of(t, "type"), format = attr_of(t, "format", "ascii");
    int size = 0;
    bool is_float = false, is_signed = false;
    if (!vtp_type(type, size, is_float, is_signed))
        return io_fail(ACVD_ERR_UNSUPPORTED, "VTK XML: data type " + type + " not read");
    if (format == "ascii") {
        if (t.empty) return ACVD_OK;
        const size_t end = s.find("</DataArray>", t.close);
        if (end == std::string::npos) return io_fail(ACVD_ERR_ARG, "VTK XML: unterminated DataArray");
        std::istringstream in(s.substr(t.close, end - t.close));
        std::string tok;
        while (in >> tok) {
            char* e = nullptr;
            if (dv) dv->push_back(std::strtod(tok.c_str(), &e));
            else iv->push_back((int64_t)std::strtoll(tok.c_str(), &e, 10));
            if (!e || *e) return io_fail(ACVD_ERR_ARG, "VTK XML: bad ascii value '" + tok + "'");
        }
        return ACVD_OK;
    }
    std::string block, raw;
    if (format == "binary") {
        const size_t end = s.find("</DataArray>", t.close);
        if (t.empty || end == std::string::npos) return io_fail(ACVD_ERR_ARG, "VTK XML: unterminated DataArray");
        if (!b64_decode(s.data() + t.close, end - t.close, block))
            return io_fail(ACVD_ERR_ARG, "VTK XML: bad base64 data");
    } else if (format == "appended") {
        const size_t off = (size_t)std::strtoull(attr_of(t, "offset", "0").c_str(), nullptr, 10);
        if (off > f.appended.size()) return io_fail(ACVD_ERR_ARG, "VTK XML: appended offset past the data");
        if (f.appended_b64) {
            auto nx = std::upper_bound(f.offsets.begin(), f.offsets.end(), off);
            const size_t stop = nx == f.offsets.end() ? f.appended.size() : *nx;
            if (!b64_decode(f.appended.data() + off, stop - off, block))
                return io_fail(ACVD_ERR_ARG, "VTK XML: bad base64 data");
        } else {
            block.assign(f.appended, off, std::string::npos);
        }
    } else {
        return io_fail(ACVD_ERR_UNSUPPORTED, "VTK XML: DataArray format " + format + " not read");
    }
    if (!vtp_block(f, (const unsigned char*)block.data(), block.size(), raw))
        return io_fail(ACVD_ERR_ARG, "VTK XML: corrupt or truncated binary data");
    const size_t n = raw.size() / (size_t)size;
    const unsigned char* p = (const unsigned char*)raw.data();
    for (size_t i = 0; i < n; i++, p += size) {
        double d = 0.0;
        int64_t v = 0;
        if (is_float) {
            d = size == 4 ? (double)load_scalar<float>(p, f.little) : load_scalar<double>(p, f.little);
            v = (int64_t)d;
        } else if (size == 1) {
            v = is_signed ? (int64_t)(int8_t)p[0] : (int64_t)p[0];
        } else if (size == 2) {
            v = is_signed ? (int64_t)load_scalar<int16_t>(p, f.little) : (int64_t)load_scalar<uint16_t>(p, f.little);
        } else if (size == 4) {
            v = is_signed ? (int64_t)load_scalar<int32_t>(p, f.little) : (int64_t)load_scalar<uint32_t>(p, f.little);
        } else {
            v = is_signed ? load_scalar<int64_t>(p, f.little) : (int64_t)load_scalar<uint64_t>(p, f.little);
        }
        if (dv) dv->push_back(is_float ? d : (double)v);
        else iv->push_back(v);
    }
    return ACVD_OK;
}

// the first DataArray in [from, stop) whose Name is `name` (any name when null)
bool vtp_find_array(const std::string& s, size_t from, size_t stop, const char* name, XmlTag& out) {
    XmlTag t;
    size_t at = from;
    while (next_tag(s, at, stop, t)) {
        at = t.close;
        if (t.name == "DataArray" && (!name || attr_of(t, "Name") == name)) {
            out = t;
            return true;
        }
    }
    return false;
}

int read_vtp(const std::string& s, MeshData& m) {
    VtpFile f;
    XmlTag t;
    size_t at = 0;
    bool found = false;
    const size_t app = s.find("<AppendedData");
    const size_t stop = app == std::string::npos ? s.size() : app;
    while (next_tag(s, at, stop, t)) {
        at = t.close;
        if (t.name == "VTKFile") {
            found = true;
            break;
        }
    }
    if (!found) return io_fail(ACVD_ERR_ARG, "not a VTK XML file");
    if (attr_of(t, "type") != "PolyData") return io_fail(ACVD_ERR_UNSUPPORTED, "VTK XML: not a PolyData file");
    f.little = attr_of(t, "byte_order", "LittleEndian") != "BigEndian";
    const std::string ht = attr_of(t, "header_type", "UInt32");
    if (ht != "UInt32" && ht != "UInt64") return io_fail(ACVD_ERR_UNSUPPORTED, "VTK XML: header_type " + ht);
    f.header_bytes = ht == "UInt64" ? 8 : 4;
    const std::string comp = attr_of(t, "compressor");
    if (!comp.empty() && comp != "vtkZLibDataCompressor")
        return io_fail(ACVD_ERR_UNSUPPORTED, "VTK XML: compressor " + comp + " not read (zlib only)");
    f.zlib = !comp.empty();
    if (app != std::string::npos) {
        XmlTag a;
        if (!next_tag(s, app, s.size(), a)) return io_fail(ACVD_ERR_ARG, "VTK XML: bad AppendedData");
        const size_t mark = s.find('_', a.close);
        if (mark == std::string::npos) return io_fail(ACVD_ERR_ARG, "VTK XML: AppendedData without '_'");
        f.appended_b64 = attr_of(a, "encoding", "raw") == "base64";
        if (f.appended_b64) {
            const size_t end = s.find('<', mark + 1);
            f.appended = s.substr(mark + 1, (end == std::string::npos ? s.size() : end) - mark - 1);
        } else {
            f.appended = s.substr(mark + 1);
        }
        XmlTag d;
        size_t k = 0;
        while (next_tag(s, k, stop, d)) {
            k = d.close;
            if (d.name == "DataArray" && attr_of(d, "format") == "appended")
                f.offsets.push_back((size_t)std::strtoull(attr_of(d, "offset", "0").c_str(), nullptr, 10));
        }
        std::sort(f.offsets.begin(), f.offsets.end());
    }
    // pieces
    int pieces = 0;
    while (next_tag(s, at, stop, t)) {
        at = t.close;
        if (t.name != "Piece") continue;
        pieces++;
        const size_t pend_raw = s.find("</Piece>", t.close);
        const size_t pend = pend_raw == std::string::npos || pend_raw > stop ? stop : pend_raw;
        if (std::strtoll(attr_of(t, "NumberOfStrips", "0").c_str(), nullptr, 10) > 0)
            return io_fail(ACVD_ERR_UNSUPPORTED, "VTK XML: triangle strips are not read");
        const int64_t np = std::strtoll(attr_of(t, "NumberOfPoints", "0").c_str(), nullptr, 10);
        const int64_t npoly = std::strtoll(attr_of(t, "NumberOfPolys", "0").c_str(), nullptr, 10);
        const int64_t base = (int64_t)m.xyz.size() / 3;
        std::vector<double> pts;
        const size_t ptag = s.find("<Points", t.close);
        XmlTag arr;
        if (np > 0) {
            if (ptag == std::string::npos || ptag > pend || !vtp_find_array(s, ptag, pend, nullptr, arr))
                return io_fail(ACVD_ERR_ARG, "VTK XML: a Piece without Points");
            if (int rc = vtp_array(s, f, arr, &pts, nullptr)) return rc;
            if ((int64_t)pts.size() != 3 * np) return io_fail(ACVD_ERR_ARG, "VTK XML: Points count mismatch");
        }
        m.xyz.insert(m.xyz.end(), pts.begin(), pts.end());
        if (npoly == 0) continue;
        const size_t ytag = s.find("<Polys", t.close);
        if (ytag == std::string::npos || ytag > pend) return io_fail(ACVD_ERR_ARG, "VTK XML: Polys missing");
        std::vector<int64_t> conn, offs;
        if (!vtp_find_array(s, ytag, pend, "connectivity", arr)) return io_fail(ACVD_ERR_ARG, "VTK XML: no connectivity");
        if (int rc = vtp_array(s, f, arr, nullptr, &conn)) return rc;
        if (!vtp_find_array(s, ytag, pend, "offsets", arr)) return io_fail(ACVD_ERR_ARG, "VTK XML: no offsets");
        if (int rc = vtp_array(s, f, arr, nullptr, &offs)) return rc;
        if ((int64_t)offs.size() != npoly) return io_fail(ACVD_ERR_ARG, "VTK XML: Polys count mismatch");
        int64_t prev = 0;
        std::vector<int64_t> poly;
        for (int64_t e : offs) {
            if (e < prev || e > (int64_t)conn.size()) return io_fail(ACVD_ERR_ARG, "VTK XML: bad Polys offsets");
            poly.assign(conn.begin() + prev, conn.begin() + e);
            for (int64_t& v : poly) {
                if (v < 0 || v >= np) return io_fail(ACVD_ERR_ARG, "VTK XML: a face refers to a missing point");
                v += base;
            }
            if (int rc = add_polygon(m, poly)) return rc;
            prev = e;
        }
    }
    if (!pieces) return io_fail(ACVD_ERR_ARG, "VTK XML: no Piece");
    return check_faces(m);
}

// ---------------------------------------------------------------- MetaImage density
// The custom density of vtkDiscreteRemeshing::SamplingPreProcessing
// (DiscreteRemeshing/vtkDiscreteRemeshing.h:603-640): a scalar volume read from a
// MetaImage file (.mhd header with its data file, or .mha with the data inline; raw or
// zlib-compressed), sampled at each vertex in the voxel whose cell holds it
// (vtkImageData::ComputeStructuredCoordinates: i = floor((x - origin) / spacing), the last
// cell at the upper face; outside the volume the value is 0), and mapped to
// max(max_density - value * factor, min_density).  Written from MetaIO's published header
// keys: NDims, DimSize, ElementSpacing, Offset / Origin / Position, ElementType,
// ElementNumberOfChannels, ElementByteOrderMSB / BinaryDataByteOrderMSB,
// CompressedData, HeaderSize and ElementDataFile (LOCAL or a file name).
int read_metaimage(const std::string& path, std::vector<int64_t>& dim, std::vector<double>& origin,
                   std::vector<double>& spacing, std::vector<double>& values) {
    std::string buf;
    if (!read_all(path.c_str(), buf)) return io_fail(ACVD_ERR_ARG, "cannot read " + path);
    std::map<std::string, std::string> kv;
    size_t pos = 0, data_at = std::string::npos;
    while (pos < buf.size()) {
        const size_t eol = buf.find('\n', pos);
        const size_t end = eol == std::string::npos ? buf.size() : eol;
        std::string line = buf.substr(pos, end - pos);
        pos = end + 1;
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        auto trim = [](std::string s) {
            const size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
            return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
        };
        const std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
        kv[key] = val;
        if (key == "ElementDataFile") {
            data_at = pos;
            break;
        }
    }
    if (data_at == std::string::npos) return io_fail(ACVD_ERR_ARG, "MetaImage: no ElementDataFile in " + path);
    auto get = [&](const char* k) { auto it = kv.find(k); return it == kv.end() ? std::string() : it->second; };
    auto numbers = [](const std::string& s) {
        std::vector<double> v;
        std::istringstream in(s);
        double x;
        while (in >> x) v.push_back(x);
        return v;
    };
    const int nd = std::atoi(get("NDims").c_str());
    if (nd < 1 || nd > 3) return io_fail(ACVD_ERR_UNSUPPORTED, "MetaImage: NDims must be 1 to 3");
    const std::vector<double> ds = numbers(get("DimSize"));
    if ((int)ds.size() < nd) return io_fail(ACVD_ERR_ARG, "MetaImage: DimSize");
    dim.assign(3, 1);
    origin.assign(3, 0.0);
    spacing.assign(3, 1.0);
    // each extent and the voxel count are bounded (2^31 per axis, 2^36 voxels) so
    // that the byte count below cannot wrap
    constexpr double kMaxExtent = 2147483648.0;
    constexpr uint64_t kMaxVoxels = 1ull << 36;
    for (int i = 0; i < nd; i++) {
        if (!(ds[i] >= 1 && ds[i] <= kMaxExtent)) return io_fail(ACVD_ERR_ARG, "MetaImage: DimSize");
        dim[i] = (int64_t)ds[i];
    }
    if ((uint64_t)dim[0] * (uint64_t)dim[1] > kMaxVoxels ||
        (uint64_t)dim[0] * (uint64_t)dim[1] * (uint64_t)dim[2] > kMaxVoxels)
        return io_fail(ACVD_ERR_ARG, "MetaImage: DimSize too large");
    std::vector<double> sp = numbers(get("ElementSpacing"));
    if (sp.empty()) sp = numbers(get("ElementSize"));
    for (int i = 0; i < nd && i < (int)sp.size(); i++) spacing[i] = sp[i];
    std::vector<double> org = numbers(get("Offset"));
    if (org.empty()) org = numbers(get("Origin"));
    if (org.empty()) org = numbers(get("Position"));
    for (int i = 0; i < nd && i < (int)org.size(); i++) origin[i] = org[i];
    const std::string et = get("ElementType");
    int size = 0;
    bool is_float = false, is_signed = true;
    if (et == "MET_CHAR") size = 1;
    else if (et == "MET_UCHAR") { size = 1; is_signed = false; }
    else if (et == "MET_SHORT") size = 2;
    else if (et == "MET_USHORT") { size = 2; is_signed = false; }
    else if (et == "MET_INT" || et == "MET_LONG") size = 4;
    else if (et == "MET_UINT" || et == "MET_ULONG") { size = 4; is_signed = false; }
    else if (et == "MET_LONG_LONG") size = 8;
    else if (et == "MET_ULONG_LONG") { size = 8; is_signed = false; }
    else if (et == "MET_FLOAT") { size = 4; is_float = true; }
    else if (et == "MET_DOUBLE") { size = 8; is_float = true; }
    else return io_fail(ACVD_ERR_UNSUPPORTED, "MetaImage: ElementType " + et);
    const long long channels_in = std::atoll(get("ElementNumberOfChannels").c_str());
    if (channels_in > 1024) return io_fail(ACVD_ERR_ARG, "MetaImage: ElementNumberOfChannels too large");
    const int channels = (int)std::max(1LL, channels_in);
    std::string msb = get("ElementByteOrderMSB");
    if (msb.empty()) msb = get("BinaryDataByteOrderMSB");
    const bool little = !(msb == "True" || msb == "true" || msb == "1");
    const std::string cd = get("CompressedData");
    const bool compressed = cd == "True" || cd == "true" || cd == "1";
    const size_t count = (size_t)(dim[0] * dim[1] * dim[2]);
    const size_t nbytes = count * (size_t)channels * (size_t)size;
    std::string file = get("ElementDataFile"), data;
    const char* p = nullptr;
    size_t avail = 0;
    if (file == "LOCAL") {
        p = buf.data() + data_at;
        avail = buf.size() - data_at;
    } else {
        if (file.find("%") != std::string::npos || file == "LIST")
            return io_fail(ACVD_ERR_UNSUPPORTED, "MetaImage: lists of data files are not read");
        const size_t slash = path.find_last_of('/');
        if (file[0] != '/' && slash != std::string::npos) file = path.substr(0, slash + 1) + file;
        if (!read_all(file.c_str(), data)) return io_fail(ACVD_ERR_ARG, "cannot read " + file);
        const long long hs = std::atoll(get("HeaderSize").c_str());
        size_t skip = 0;
        if (hs > 0) skip = (size_t)hs;
        else if (hs == -1 && !compressed && data.size() >= nbytes) skip = data.size() - nbytes;   // data at the end
        if (skip > data.size()) return io_fail(ACVD_ERR_ARG, "MetaImage: HeaderSize past the data");
        p = data.data() + skip;
        avail = data.size() - skip;
    }
    std::string raw;
    if (compressed) {
        if (!zlib_inflate((const unsigned char*)p, avail, nbytes, raw))
            return io_fail(ACVD_ERR_ARG, "MetaImage: corrupt compressed data");
    } else {
        if (avail < nbytes) return io_fail(ACVD_ERR_ARG, "MetaImage: data shorter than DimSize says");
        raw.assign(p, nbytes);
    }
    values.resize(count);
    const unsigned char* q = (const unsigned char*)raw.data();
    for (size_t i = 0; i < count; i++, q += (size_t)channels * size) {   // first component
        double v;
        if (is_float) v = size == 4 ? (double)load_scalar<float>(q, little) : load_scalar<double>(q, little);
        else if (size == 1) v = is_signed ? (double)(int8_t)q[0] : (double)q[0];
        else if (size == 2) v = is_signed ? (double)load_scalar<int16_t>(q, little) : (double)load_scalar<uint16_t>(q, little);
        else if (size == 4) v = is_signed ? (double)load_scalar<int32_t>(q, little) : (double)load_scalar<uint32_t>(q, little);
        else v = is_signed ? (double)load_scalar<int64_t>(q, little) : (double)load_scalar<uint64_t>(q, little);
        values[i] = v;
    }
    return ACVD_OK;
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

// VTK XML PolyData: inline base64 blocks with a UInt64 byte-count header, little endian,
// float32 points (the float vtkPoints of vtkSurface), Int64 connectivity and offsets
std::string write_vtp(const double* xyz, int64_t nv, const int32_t* tri, int64_t nf) {
    auto block = [](const std::string& raw) {
        std::string b;
        store_scalar<uint64_t>(b, (uint64_t)raw.size(), true);
        b += raw;
        std::string enc;
        b64_encode(b, enc);
        return enc;
    };
    std::string pts, conn, offs;
    for (int64_t i = 0; i < 3 * nv; i++) store_scalar<float>(pts, (float)xyz[i], true);
    for (int64_t i = 0; i < 3 * nf; i++) store_scalar<int64_t>(conn, (int64_t)tri[i], true);
    for (int64_t f = 1; f <= nf; f++) store_scalar<int64_t>(offs, 3 * f, true);
    std::string out = "<?xml version=\"1.0\"?>\n"
                      "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
                      "  <PolyData>\n    <Piece NumberOfPoints=\"" + std::to_string(nv) +
                      "\" NumberOfVerts=\"0\" NumberOfLines=\"0\" NumberOfStrips=\"0\" NumberOfPolys=\"" +
                      std::to_string(nf) + "\">\n      <Points>\n"
                      "        <DataArray type=\"Float32\" Name=\"Points\" NumberOfComponents=\"3\" format=\"binary\">\n"
                      "          " + block(pts) + "\n        </DataArray>\n      </Points>\n      <Polys>\n"
                      "        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"binary\">\n"
                      "          " + block(conn) + "\n        </DataArray>\n"
                      "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"binary\">\n"
                      "          " + block(offs) + "\n        </DataArray>\n      </Polys>\n    </Piece>\n"
                      "  </PolyData>\n</VTKFile>\n";
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
    else if (name.find(".vtp") != std::string::npos) rc = read_vtp(buf, m);
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

int acvd_density_indicator(const char* image_path, int64_t n_vertices, const double* xyz, double max_density,
                           double min_density, double factor, double* indicator) {
    if (!image_path || n_vertices < 0 || (n_vertices && (!xyz || !indicator)))
        return io_fail(ACVD_ERR_ARG, "null or negative argument");
    const std::string name = lower(image_path);
    if (name.find(".mnc") != std::string::npos)
        return io_fail(ACVD_ERR_UNSUPPORTED, "MINC density images are not read (MetaImage only)");
    std::vector<int64_t> dim;
    std::vector<double> origin, spacing, values;
    if (int rc = read_metaimage(image_path, dim, origin, spacing, values)) return rc;
    for (int64_t i = 0; i < n_vertices; i++) {
        int64_t ijk[3];
        bool inside = true;
        for (int c = 0; c < 3; c++) {
            const double d = (xyz[3 * i + c] - origin[c]) / spacing[c];
            if (dim[c] == 1) {
                ijk[c] = 0;
                inside = inside && d == 0.0;
                continue;
            }
            if (!(d >= 0.0 && d <= (double)(dim[c] - 1))) {
                inside = false;
                ijk[c] = 0;
                continue;
            }
            ijk[c] = std::min((int64_t)std::floor(d), dim[c] - 2);   // the last cell at the upper face
        }
        const double v = inside ? values[(size_t)((ijk[2] * dim[1] + ijk[1]) * dim[0] + ijk[0])] : 0.0;
        double ind = max_density - v * factor;
        if (ind < min_density) ind = min_density;
        indicator[i] = ind;
    }
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
    else if (name.find(".vtp") != std::string::npos) out = write_vtp(xyz, n_vertices, tri, n_faces);
    else if (name.find(".off") != std::string::npos) out = write_off(xyz, n_vertices, tri, n_faces);
    else if (name.find(".obj") != std::string::npos) out = write_obj(xyz, n_vertices, tri, n_faces);
    else return io_fail(ACVD_ERR_UNSUPPORTED, std::string("unknown mesh file type: ") + path);
    std::ofstream f(path, std::ios::binary);
    if (!f) return io_fail(ACVD_ERR_ARG, std::string("cannot write ") + path);
    f.write(out.data(), (std::streamsize)out.size());
    return f ? ACVD_OK : io_fail(ACVD_ERR_ARG, std::string("write failed: ") + path);
}

}  // extern "C"
