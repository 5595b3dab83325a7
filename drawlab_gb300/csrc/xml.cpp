// Scene loading in the reference's XML format (mitsuba-style tags), replacing
// loadFromXML (src/core/parser/parser.cpp:19-387) and the plugin constructors
// it calls.  A small own XML reader builds the element tree; the interpreter
// then follows the reference's rules: properties fill the enclosing object's
// property list, objects are created with their children, `id`/`ref` pool
// shared objects, transforms compose left-multiplied in document order, and
// emitters join the scene's emitter list in the order Scene::addChild sees
// them (src/tracer/scene/scene.cpp:36-81).
//
// Supported plugins: mesh rectangle|obj, bsdf diffuse|mirror|dielectric|
// microfacet|aniso_ggx (with bitmap textures from PNG / PFM), emitter
// area|point|envmap (PFM images), camera
// virtual|perspective|opencv, integrator path|normals,
// sampler independent, rfilter gaussian|box.  Anything else is reported as
// DL_ERR_UNSUPPORTED with its location.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <list>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"
#include "scene.h"

namespace dl {
namespace {

// ---------------------------------------------------------------- XML tree
struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::unique_ptr<XNode>> children;
    int line = 0;
    const std::string* attr(const std::string& k) const {
        for (auto& a : attrs)
            if (a.first == k) return &a.second;
        return nullptr;
    }
};

[[noreturn]] void parse_fail(const std::string& file, int line, const std::string& msg) {
    throw Error(DL_ERR_PARSE, "Error while parsing \"" + file + "\": " + msg + " (at line " + std::to_string(line) + ")");
}

std::string decode_entities(const std::string& s) {
    std::string out;
    for (size_t i = 0; i < s.size(); i++) {
        if (s[i] == '&') {
            size_t e = s.find(';', i);
            if (e != std::string::npos) {
                std::string ent = s.substr(i + 1, e - i - 1);
                if (ent == "lt") { out += '<'; i = e; continue; }
                if (ent == "gt") { out += '>'; i = e; continue; }
                if (ent == "amp") { out += '&'; i = e; continue; }
                if (ent == "quot") { out += '"'; i = e; continue; }
                if (ent == "apos") { out += '\''; i = e; continue; }
            }
        }
        out += s[i];
    }
    return out;
}

struct XmlReader {
    const std::string& src;
    const std::string& file;
    size_t i = 0;
    int line = 1;
    XmlReader(const std::string& s, const std::string& f) : src(s), file(f) {}

    void adv(size_t n) {
        for (size_t k = 0; k < n && i < src.size(); k++, i++)
            if (src[i] == '\n') line++;
    }
    bool starts(const char* s) const { return src.compare(i, std::strlen(s), s) == 0; }
    void skip_ws() {
        while (i < src.size() && std::isspace((unsigned char)src[i])) adv(1);
    }
    // Skips whitespace, comments, declarations; text content is an error.
    void skip_misc() {
        for (;;) {
            skip_ws();
            if (starts("<!--")) {
                size_t e = src.find("-->", i);
                if (e == std::string::npos) parse_fail(file, line, "unterminated comment");
                adv(e + 3 - i);
            } else if (starts("<?")) {
                size_t e = src.find("?>", i);
                if (e == std::string::npos) parse_fail(file, line, "unterminated declaration");
                adv(e + 2 - i);
            } else if (starts("<!DOCTYPE")) {
                size_t e = src.find('>', i);
                if (e == std::string::npos) parse_fail(file, line, "unterminated doctype");
                adv(e + 1 - i);
            } else {
                return;
            }
        }
    }
    std::string name() {
        size_t b = i;
        while (i < src.size() && (std::isalnum((unsigned char)src[i]) || src[i] == '_' || src[i] == '-' ||
                                  src[i] == ':' || src[i] == '.'))
            adv(1);
        if (b == i) parse_fail(file, line, "expected a name");
        return src.substr(b, i - b);
    }
    std::unique_ptr<XNode> element() {
        skip_misc();
        if (i >= src.size() || src[i] != '<') parse_fail(file, line, "unexpected content");
        adv(1);
        auto n = std::make_unique<XNode>();
        n->line = line;
        n->name = name();
        for (;;) {
            skip_ws();
            if (starts("/>")) {
                adv(2);
                return n;
            }
            if (starts(">")) {
                adv(1);
                break;
            }
            std::string k = name();
            skip_ws();
            if (i >= src.size() || src[i] != '=') parse_fail(file, line, "expected '=' after attribute " + k);
            adv(1);
            skip_ws();
            if (i >= src.size() || (src[i] != '"' && src[i] != '\'')) parse_fail(file, line, "expected a quoted value");
            char q = src[i];
            adv(1);
            size_t e = src.find(q, i);
            if (e == std::string::npos) parse_fail(file, line, "unterminated attribute value");
            std::string v = decode_entities(src.substr(i, e - i));
            adv(e + 1 - i);
            for (auto& a : n->attrs)
                if (a.first == k) parse_fail(file, line, "duplicate attribute " + k);
            n->attrs.push_back({k, v});
        }
        for (;;) {
            skip_misc();
            if (starts("</")) {
                adv(2);
                std::string nm = name();
                if (nm != n->name) parse_fail(file, line, "mismatched closing tag </" + nm + ">");
                skip_ws();
                if (i >= src.size() || src[i] != '>') parse_fail(file, line, "expected '>'");
                adv(1);
                return n;
            }
            if (i >= src.size()) parse_fail(file, line, "unterminated element <" + n->name + ">");
            n->children.push_back(element());
        }
    }
};

// ------------------------------------------------------------ properties
struct M4 {
    float m[4][4];
    static M4 identity() {
        M4 r;
        std::memset(r.m, 0, sizeof(r.m));
        for (int k = 0; k < 4; k++) r.m[k][k] = 1.f;
        return r;
    }
    M4 operator*(const M4& b) const {
        M4 r;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                float s = 0;
                for (int k = 0; k < 4; k++) s += m[i][k] * b.m[k][j];
                r.m[i][j] = s;
            }
        return r;
    }
};

M4 inverse(const M4& a) {
    double m[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 8; j++) m[i][j] = j < 4 ? a.m[i][j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; c++) {
        int p = c;
        for (int r = c + 1; r < 4; r++)
            if (std::fabs(m[r][c]) > std::fabs(m[p][c])) p = r;
        if (std::fabs(m[p][c]) < 1e-30) throw Error(DL_ERR_INVALID_ARG, "singular transform");
        if (p != c)
            for (int j = 0; j < 8; j++) std::swap(m[p][j], m[c][j]);
        double d = m[c][c];
        for (int j = 0; j < 8; j++) m[c][j] /= d;
        for (int r = 0; r < 4; r++)
            if (r != c) {
                double f = m[r][c];
                for (int j = 0; j < 8; j++) m[r][j] -= f * m[c][j];
            }
    }
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.m[i][j] = (float)m[i][j + 4];
    return r;
}

enum PType { P_BOOL, P_INT, P_FLOAT, P_STRING, P_POINT, P_VECTOR, P_COLOR, P_TRANSFORM };

struct Prop {
    PType type;
    bool b = false;
    int i = 0;
    float f = 0;
    std::string s;
    float v[3] = {0, 0, 0};
    M4 t = M4::identity();
};

struct Obj;

struct Props {
    std::map<std::string, Prop> p;
    std::string file;
    int line = 0;
    const Prop* get(const std::string& k, PType t) const {
        auto it = p.find(k);
        if (it == p.end()) return nullptr;
        if (it->second.type != t)
            throw Error(DL_ERR_PARSE, "property \"" + k + "\" has the wrong type (line " + std::to_string(line) + ")");
        return &it->second;
    }
    [[noreturn]] void missing(const std::string& k) const {
        throw Error(DL_ERR_PARSE, "Error while parsing \"" + file + "\": property \"" + k +
                                      "\" is required (at line " + std::to_string(line) + ")");
    }
    float f(const std::string& k, float d) const {
        auto q = get(k, P_FLOAT);
        return q ? q->f : d;
    }
    float f(const std::string& k) const {  // required
        auto q = get(k, P_FLOAT);
        if (!q) missing(k);
        return q->f;
    }
    int i(const std::string& k, int d) const {
        auto q = get(k, P_INT);
        return q ? q->i : d;
    }
    bool b(const std::string& k, bool d) const {
        auto q = get(k, P_BOOL);
        return q ? q->b : d;
    }
    std::string s(const std::string& k) const {
        auto q = get(k, P_STRING);
        if (!q) missing(k);
        return q->s;
    }
    void vec(const std::string& k, PType t, float* out, const float* d) const {
        auto q = get(k, t);
        if (!q && !d) missing(k);
        const float* src = q ? q->v : d;
        for (int j = 0; j < 3; j++) out[j] = src[j];
    }
    M4 transform(const std::string& k) const {
        auto q = get(k, P_TRANSFORM);
        return q ? q->t : M4::identity();
    }
};

enum ObjKind { O_SCENE, O_MESH, O_BSDF, O_EMITTER, O_CAMERA, O_INTEGRATOR, O_SAMPLER, O_RFILTER, O_TEXTURE };

struct Obj {
    ObjKind kind;
    std::string type;
    std::string name;  // the "name" attribute (texture slots)
    Props props;
    std::vector<Obj*> children;
    int line = 0;
};

float to_float(const std::string& s, const std::string& file, int line) {
    char* end = nullptr;
    float r = std::strtof(s.c_str(), &end);
    if (s.empty() || *end != '\0') parse_fail(file, line, "could not parse floating point value \"" + s + "\"");
    return r;
}
std::vector<std::string> tokenize(const std::string& s) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : s) {
        if (c == ',' || c == ' ' || c == '\t' || c == '\n' || c == '\r') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}
void to_vec3(const std::string& s, float* v, const std::string& file, int line, bool allow_scalar = false) {
    auto t = tokenize(s);
    if (allow_scalar && t.size() == 1) {
        v[0] = v[1] = v[2] = to_float(t[0], file, line);
        return;
    }
    if (t.size() != 3) parse_fail(file, line, "expected 3 values in \"" + s + "\"");
    for (int k = 0; k < 3; k++) v[k] = to_float(t[k], file, line);
}

struct Interp {
    std::string file, dir;
    std::vector<std::unique_ptr<Obj>> pool_owner;
    std::map<std::string, Obj*> pool;
    M4 transform = M4::identity();

    const std::map<std::string, ObjKind> obj_tags{
        {"scene", O_SCENE}, {"mesh", O_MESH}, {"shape", O_MESH}, {"bsdf", O_BSDF}, {"emitter", O_EMITTER},
        {"camera", O_CAMERA}, {"integrator", O_INTEGRATOR}, {"sampler", O_SAMPLER}, {"rfilter", O_RFILTER},
        {"texture", O_TEXTURE}};

    void check_attrs(const XNode& n, std::vector<std::string> req, std::vector<std::string> opt = {}) {
        for (auto& a : n.attrs) {
            bool in_req = false, in_opt = false;
            for (auto& r : req) in_req |= r == a.first;
            for (auto& o : opt) in_opt |= o == a.first;
            if (!in_req && !in_opt) parse_fail(file, n.line, "unexpected attribute \"" + a.first + "\" in \"" + n.name + "\"");
        }
        for (auto& r : req)
            if (!n.attr(r)) parse_fail(file, n.line, "missing attribute \"" + r + "\" in \"" + n.name + "\"");
    }

    // parseTag of parser.cpp:147-383
    Obj* parse(const XNode& n, Props& parent, int parent_tag, bool parent_is_transform) {
        bool is_obj = obj_tags.count(n.name) > 0;
        bool is_ref = n.name == "ref";
        bool is_transform_op = n.name == "translate" || n.name == "rotate" || n.name == "scale" ||
                               n.name == "lookat" || n.name == "matrix";
        bool has_parent = parent_tag >= 0;
        if (!has_parent && !is_obj) parse_fail(file, n.line, "root element \"" + n.name + "\" must be an object");
        if (parent_is_transform != is_transform_op)
            parse_fail(file, n.line, "transform nodes can only contain transform operations");
        if (is_ref) {
            check_attrs(n, {"id"});
            auto it = pool.find(*n.attr("id"));
            if (it == pool.end()) parse_fail(file, n.line, "can't find the referred node " + *n.attr("id"));
            return it->second;
        }
        if (n.name == "transform") transform = M4::identity();
        if (!is_obj && !is_transform_op && n.name != "transform" && n.name != "boolean" && n.name != "integer" &&
            n.name != "float" && n.name != "string" && n.name != "point" && n.name != "vector" && n.name != "color")
            parse_fail(file, n.line, "unexpected tag \"" + n.name + "\"");

        Props props;
        props.file = file;
        props.line = n.line;
        std::vector<Obj*> children;
        for (auto& ch : n.children) {
            Obj* c = parse(*ch, props, is_obj ? 1 : 0, n.name == "transform");
            if (c) children.push_back(c);
        }
        if (is_obj) {
            ObjKind kind = obj_tags.at(n.name);
            if (kind == O_SCENE) {
                check_attrs(n, {}, {"name", "id", "type"});
            } else {
                check_attrs(n, {"type"}, {"name", "id"});
            }
            auto o = std::make_unique<Obj>();
            o->kind = kind;
            o->type = kind == O_SCENE ? "scene" : *n.attr("type");
            if (const std::string* nm = n.attr("name")) o->name = *nm;
            o->props = props;
            o->children = children;
            o->line = n.line;
            Obj* raw = o.get();
            pool_owner.push_back(std::move(o));
            if (const std::string* id = n.attr("id")) {
                if (!id->empty()) {
                    if (pool.count(*id)) parse_fail(file, n.line, "the node id has been used");
                    pool[*id] = raw;
                }
            }
            return raw;
        }
        // properties
        Prop pr;
        const std::string& nm = n.name;
        if (nm == "transform") {
            check_attrs(n, {"name"});
            pr.type = P_TRANSFORM;
            pr.t = transform;
            parent.p[*n.attr("name")] = pr;
        } else if (nm == "translate") {
            check_attrs(n, {"value"});
            float v[3];
            to_vec3(*n.attr("value"), v, file, n.line);
            M4 m = M4::identity();
            m.m[0][3] = v[0]; m.m[1][3] = v[1]; m.m[2][3] = v[2];
            transform = m * transform;
        } else if (nm == "scale") {
            check_attrs(n, {"value"});
            float v[3];
            to_vec3(*n.attr("value"), v, file, n.line, true);
            M4 m = M4::identity();
            m.m[0][0] = v[0]; m.m[1][1] = v[1]; m.m[2][2] = v[2];
            transform = m * transform;
        } else if (nm == "rotate") {
            check_attrs(n, {"angle", "axis"});
            float ang = to_float(*n.attr("angle"), file, n.line) * (3.14159265358979323846f / 180.0f);
            float a[3];
            to_vec3(*n.attr("axis"), a, file, n.line);
            float c = std::cos(ang), s = std::sin(ang), x = a[0], y = a[1], z = a[2];
            M4 m = M4::identity();
            m.m[0][0] = c + (1 - c) * x * x; m.m[0][1] = (1 - c) * x * y - s * z; m.m[0][2] = (1 - c) * x * z + s * y;
            m.m[1][0] = (1 - c) * y * x + s * z; m.m[1][1] = c + (1 - c) * y * y; m.m[1][2] = (1 - c) * y * z - s * x;
            m.m[2][0] = (1 - c) * z * x - s * y; m.m[2][1] = (1 - c) * z * y + s * x; m.m[2][2] = c + (1 - c) * z * z;
            transform = m * transform;
        } else if (nm == "matrix") {
            check_attrs(n, {"value"});
            auto t = tokenize(*n.attr("value"));
            if (t.size() != 16) parse_fail(file, n.line, "expected 16 values");
            M4 m;
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) m.m[r][c] = to_float(t[4 * r + c], file, n.line);
            transform = m * transform;
        } else if (nm == "lookat") {
            check_attrs(n, {"origin", "target", "up"});
            float o[3], tg[3], up[3];
            to_vec3(*n.attr("origin"), o, file, n.line);
            to_vec3(*n.attr("target"), tg, file, n.line);
            to_vec3(*n.attr("up"), up, file, n.line);
            auto nrm = [](float* v) {
                float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                for (int k = 0; k < 3; k++) v[k] /= l;
            };
            auto crs = [](const float* a, const float* b, float* r) {
                r[0] = a[1] * b[2] - a[2] * b[1];
                r[1] = a[2] * b[0] - a[0] * b[2];
                r[2] = a[0] * b[1] - a[1] * b[0];
            };
            float dir[3] = {tg[0] - o[0], tg[1] - o[1], tg[2] - o[2]};
            nrm(dir);
            nrm(up);
            float left[3], nup[3];
            crs(up, dir, left);
            nrm(left);
            crs(dir, left, nup);
            nrm(nup);
            M4 m = M4::identity();
            for (int k = 0; k < 3; k++) {
                m.m[k][0] = left[k];
                m.m[k][1] = nup[k];
                m.m[k][2] = dir[k];
                m.m[k][3] = o[k];
            }
            transform = m * transform;
        } else {
            check_attrs(n, {"name", "value"});
            const std::string& v = *n.attr("value");
            if (nm == "string") {
                pr.type = P_STRING;
                pr.s = v;
            } else if (nm == "float") {
                pr.type = P_FLOAT;
                pr.f = to_float(v, file, n.line);
            } else if (nm == "integer") {
                pr.type = P_INT;
                char* end = nullptr;
                long r = std::strtol(v.c_str(), &end, 10);
                if (v.empty() || *end != '\0') parse_fail(file, n.line, "could not parse integer value \"" + v + "\"");
                pr.i = (int)r;
            } else if (nm == "boolean") {
                pr.type = P_BOOL;
                std::string lv;
                for (char c : v) lv += (char)std::tolower((unsigned char)c);
                if (lv == "true") pr.b = true;
                else if (lv == "false") pr.b = false;
                else parse_fail(file, n.line, "could not parse boolean value \"" + v + "\"");
            } else {
                pr.type = nm == "point" ? P_POINT : (nm == "vector" ? P_VECTOR : P_COLOR);
                to_vec3(v, pr.v, file, n.line);
            }
            parent.p[*n.attr("name")] = pr;
        }
        return nullptr;
    }
};

// -------------------------------------------------------------- geometry
struct MeshData {
    std::vector<float> V, N, UV;
    std::vector<uint32_t> F;
};

void apply_transform(MeshData& m, const M4& T) {
    M4 nt = inverse(T);
    for (size_t k = 0; k + 2 < m.V.size(); k += 3) {
        float p[4] = {m.V[k], m.V[k + 1], m.V[k + 2], 1.f}, r[4];
        for (int i = 0; i < 4; i++) r[i] = T.m[i][0] * p[0] + T.m[i][1] * p[1] + T.m[i][2] * p[2] + T.m[i][3] * p[3];
        m.V[k] = r[0] / r[3];
        m.V[k + 1] = r[1] / r[3];
        m.V[k + 2] = r[2] / r[3];
    }
    for (size_t k = 0; k + 2 < m.N.size(); k += 3) {
        float n[3] = {m.N[k], m.N[k + 1], m.N[k + 2]}, r[3];
        // inverse transpose
        for (int i = 0; i < 3; i++) r[i] = nt.m[0][i] * n[0] + nt.m[1][i] * n[1] + nt.m[2][i] * n[2];
        m.N[k] = r[0];
        m.N[k + 1] = r[1];
        m.N[k + 2] = r[2];
    }
}

// Wavefront OBJ: one vertex per distinct (position, texcoord, normal) index
// triple in order of first use, faces fan-triangulated (the layout
// tinyobjloader gives src/tracer/mesh/obj.cpp).
MeshData load_obj(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw Error(DL_ERR_IO, "cannot open OBJ file \"" + path + "\"");
    std::vector<float> P, T, Nn;
    MeshData m;
    std::map<std::tuple<int, int, int>, uint32_t> cache;
    bool any_n = false, any_t = false;
    std::vector<std::tuple<int, int, int>> verts;
    std::string line;
    int ln = 0;
    auto fix = [](int idx, size_t count) { return idx < 0 ? (int)count + idx : idx - 1; };
    while (std::getline(in, line)) {
        ln++;
        std::istringstream ss(line);
        std::string tag;
        if (!(ss >> tag)) continue;
        if (tag == "v") {
            float x, y, z;
            ss >> x >> y >> z;
            P.insert(P.end(), {x, y, z});
        } else if (tag == "vn") {
            float x, y, z;
            ss >> x >> y >> z;
            Nn.insert(Nn.end(), {x, y, z});
        } else if (tag == "vt") {
            float x = 0, y = 0;
            ss >> x >> y;
            T.insert(T.end(), {x, y});
        } else if (tag == "f") {
            std::vector<uint32_t> poly;
            std::string tok;
            while (ss >> tok) {
                int vi = 0, ti = 0, ni = 0;
                int* slots[3] = {&vi, &ti, &ni};
                int s = 0;
                std::string cur;
                for (size_t k = 0; k <= tok.size(); k++) {
                    if (k == tok.size() || tok[k] == '/') {
                        if (!cur.empty() && s < 3) *slots[s] = std::atoi(cur.c_str());
                        cur.clear();
                        s++;
                    } else {
                        cur += tok[k];
                    }
                }
                int v = fix(vi, P.size() / 3), t = ti ? fix(ti, T.size() / 2) : -1, n = ni ? fix(ni, Nn.size() / 3) : -1;
                if (v < 0 || (size_t)v >= P.size() / 3) throw Error(DL_ERR_PARSE, path + ": bad vertex index at line " + std::to_string(ln));
                auto key = std::make_tuple(v, t, n);
                auto it = cache.find(key);
                uint32_t id;
                if (it == cache.end()) {
                    id = (uint32_t)verts.size();
                    cache[key] = id;
                    verts.push_back(key);
                    any_n |= n >= 0;
                    any_t |= t >= 0;
                } else {
                    id = it->second;
                }
                poly.push_back(id);
            }
            for (size_t k = 1; k + 1 < poly.size(); k++) m.F.insert(m.F.end(), {poly[0], poly[k], poly[k + 1]});
        }
    }
    for (auto& vt : verts) {
        int v = std::get<0>(vt), t = std::get<1>(vt), n = std::get<2>(vt);
        m.V.insert(m.V.end(), {P[3 * v], P[3 * v + 1], P[3 * v + 2]});
        if (any_n) {
            if (n >= 0 && (size_t)n < Nn.size() / 3) m.N.insert(m.N.end(), {Nn[3 * n], Nn[3 * n + 1], Nn[3 * n + 2]});
            else m.N.insert(m.N.end(), {0.f, 0.f, 0.f});
        }
        if (any_t) {
            if (t >= 0 && (size_t)t < T.size() / 2) m.UV.insert(m.UV.end(), {T[2 * t], T[2 * t + 1]});
            else m.UV.insert(m.UV.end(), {0.f, 0.f});
        }
    }
    return m;
}

// rectangle shape (src/tracer/mesh/rectangle.cpp:11-40)
MeshData make_rectangle(const Props& p) {
    float pos[3], v0[3], v1[3];
    p.vec("pos", P_VECTOR, pos, nullptr);
    p.vec("v0", P_VECTOR, v0, nullptr);
    p.vec("v1", P_VECTOR, v1, nullptr);
    float n[3] = {v0[1] * v1[2] - v0[2] * v1[1], v0[2] * v1[0] - v0[0] * v1[2], v0[0] * v1[1] - v0[1] * v1[0]};
    float l2 = 0;
    l2 += n[0] * n[0];
    l2 += n[1] * n[1];
    l2 += n[2] * n[2];
    float l = std::sqrt(l2);
    for (float& c : n) c /= l;
    MeshData m;
    float pts[4][3];
    for (int k = 0; k < 3; k++) {
        pts[0][k] = pos[k];
        pts[1][k] = pos[k] + v0[k];
        pts[2][k] = pos[k] + v1[k];
        pts[3][k] = pos[k] + v0[k] + v1[k];
    }
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 3; k++) {
            m.V.push_back(pts[i][k]);
            m.N.push_back(n[k]);
        }
    m.UV = {1, 0, 1, 1, 0, 0, 0, 1};
    m.F = {0, 1, 2, 3, 2, 1};
    return m;
}

// A <texture type="bitmap"> child: the image (PNG or PFM, resolved against
// the scene file's directory) in the texel order the reference uploads
// (src/tracer/texture/bitmap.cpp:60-98): 8-bit images as read (top row at
// t = 0), float images flipped (bottom row at t = 0).
dl_texture_desc load_texture(const Obj& t, const std::string& dir, std::list<std::vector<float>>& store) {
    if (t.type != "bitmap")
        throw Error(DL_ERR_UNSUPPORTED, "texture type \"" + t.type + "\" is not supported (line " +
                                            std::to_string(t.line) + ")");
    std::string fn = t.props.s("filename");
    if (!fn.empty() && fn[0] != '/') fn = dir + "/" + fn;
    int w = 0, h = 0;
    bool is_float = false;
    std::vector<float> img = read_image(fn, w, h, is_float);
    if (is_float)
        for (int y = 0; y < h / 2; y++)
            std::swap_ranges(img.begin() + (size_t)y * w * 3, img.begin() + (size_t)(y + 1) * w * 3,
                             img.begin() + (size_t)(h - 1 - y) * w * 3);
    store.push_back(std::move(img));
    dl_texture_desc d;
    d.rgb = store.back().data();
    d.width = w;
    d.height = h;
    return d;
}

dl_material_desc make_material(const Obj& b, const std::string& dir, std::list<std::vector<float>>& store) {
    dl_material_desc d;
    std::memset(&d, 0, sizeof(d));
    const Props& p = b.props;
    const float half[3] = {0.5f, 0.5f, 0.5f};
    // texture children by name: diffuse "albedo" (diffuse.cpp:69-73);
    // aniso_ggx "pd", "ps", "axay", "normal", "tangent" (aniso_ggx.cpp:43-57)
    const bool aniso = b.type == "aniso_ggx";
    for (Obj* c : b.children) {
        if (c->kind != O_TEXTURE) continue;
        dl_texture_desc* slot = nullptr;
        if (b.type == "diffuse" && c->name == "albedo") slot = &d.albedo_texture;
        else if (aniso && c->name == "pd") slot = &d.albedo_texture;
        else if (aniso && c->name == "ps") slot = &d.specular_texture;
        else if (aniso && c->name == "axay") slot = &d.alpha_texture;
        else if (aniso && c->name == "normal") slot = &d.normal_texture;
        else if (aniso && c->name == "tangent") slot = &d.tangent_texture;
        else
            throw Error(DL_ERR_UNSUPPORTED, "texture \"" + c->name + "\" of a " + b.type + " bsdf is not supported (line " +
                                                std::to_string(c->line) + ")");
        *slot = load_texture(*c, dir, store);
    }
    if (aniso && (d.normal_texture.rgb || d.tangent_texture.rgb) && p.b("is_tangent_space", true))
        throw Error(DL_ERR_UNSUPPORTED, "tangent-space normal / tangent maps need mesh tangents, which no mesh "
                                        "provides; set is_tangent_space to false for world-space maps (line " +
                                            std::to_string(b.line) + ")");
    if (b.type == "diffuse") {
        d.type = DL_MAT_DIFFUSE;
        p.vec("albedo", P_COLOR, d.albedo, half);
    } else if (b.type == "mirror") {
        d.type = DL_MAT_MIRROR;
    } else if (b.type == "dielectric") {
        d.type = DL_MAT_DIELECTRIC;
        d.int_ior = p.f("intIOR", 1.5046f);
        d.ext_ior = p.f("extIOR", 1.000277f);
    } else if (b.type == "microfacet") {
        d.type = DL_MAT_MICROFACET;
        d.alpha[0] = d.alpha[1] = p.f("alpha", 0.1f);
        d.int_ior = p.f("intIOR", 1.5046f);
        d.ext_ior = p.f("extIOR", 1.000277f);
        p.vec("kd", P_COLOR, d.albedo, half);
    } else if (b.type == "aniso_ggx") {
        d.type = DL_MAT_ANISO_GGX;
        p.vec("pd", P_COLOR, d.albedo, half);
        p.vec("ps", P_COLOR, d.specular, half);
        float axay[3];
        p.vec("axay", P_COLOR, axay, half);
        d.alpha[0] = axay[0];
        d.alpha[1] = axay[1];
    } else {
        throw Error(DL_ERR_UNSUPPORTED, "bsdf type \"" + b.type + "\" is not supported (line " + std::to_string(b.line) + ")");
    }
    return d;
}

}  // namespace

int load_xml_scene(dl_context* ctx, const char* path, dl_scene** out) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw Error(DL_ERR_IO, std::string("cannot open scene file \"") + path + "\"");
    std::stringstream buf;
    buf << in.rdbuf();
    std::string src = buf.str();
    std::string file = path;
    XmlReader rd(src, file);
    std::unique_ptr<XNode> root = rd.element();
    rd.skip_misc();
    if (rd.i < src.size()) parse_fail(file, rd.line, "content after the root element");

    Interp it;
    it.file = file;
    size_t slash = file.find_last_of('/');
    it.dir = slash == std::string::npos ? std::string(".") : file.substr(0, slash);
    Props top;
    Obj* scene = it.parse(*root, top, -1, false);
    if (!scene || scene->kind != O_SCENE) throw Error(DL_ERR_PARSE, "root element must be <scene>");

    std::vector<MeshData> meshdata;
    std::vector<dl_mesh_desc> mdesc;
    std::vector<dl_material_desc> mats;
    std::map<const Obj*, int> mat_index;
    std::vector<dl_light_desc> lights;
    std::list<std::vector<float>> env_images;  // stable storage for envmap texels
    dl_camera_desc cam{};
    std::memset(&cam, 0, sizeof(cam));
    bool have_cam = false, have_integrator = false, have_sampler = false;
    uint32_t integrator_flags = 0;
    int spp = 1, filter = DL_FILTER_GAUSSIAN;
    auto add_material = [&](const Obj* b) -> int {
        auto f = mat_index.find(b);
        if (f != mat_index.end()) return f->second;
        mats.push_back(make_material(*b, it.dir, env_images));
        mat_index[b] = (int)mats.size() - 1;
        return (int)mats.size() - 1;
    };
    Obj default_bsdf;
    default_bsdf.kind = O_BSDF;
    default_bsdf.type = "diffuse";
    for (Obj* c : scene->children) {
        switch (c->kind) {
            case O_MESH: {
                MeshData md;
                if (c->type == "rectangle") {
                    md = make_rectangle(c->props);
                } else if (c->type == "obj") {
                    std::string fn = c->props.s("filename");
                    if (!fn.empty() && fn[0] != '/') fn = it.dir + "/" + fn;
                    md = load_obj(fn);
                    apply_transform(md, c->props.transform("toWorld"));
                } else {
                    throw Error(DL_ERR_UNSUPPORTED, "mesh type \"" + c->type + "\" is not supported");
                }
                const Obj* bsdf = nullptr;
                const Obj* emitter = nullptr;
                for (Obj* ch : c->children) {
                    if (ch->kind == O_BSDF) {
                        if (bsdf) throw Error(DL_ERR_PARSE, "Mesh: tried to register multiple BSDF instances!");
                        bsdf = ch;
                    } else if (ch->kind == O_EMITTER) {
                        if (emitter) throw Error(DL_ERR_PARSE, "Mesh: tried to register multiple Emitter instances!");
                        emitter = ch;
                    } else {
                        throw Error(DL_ERR_PARSE, "Mesh::addChild: unsupported child");
                    }
                }
                meshdata.push_back(std::move(md));
                dl_mesh_desc d;
                std::memset(&d, 0, sizeof(d));
                d.material = add_material(bsdf ? bsdf : &default_bsdf);
                d.light = -1;
                if (emitter) {
                    if (emitter->type != "area")
                        throw Error(DL_ERR_UNSUPPORTED, "emitter \"" + emitter->type + "\" cannot be attached to a mesh");
                    dl_light_desc L;
                    std::memset(&L, 0, sizeof(L));
                    L.type = DL_LIGHT_AREA;
                    L.mesh = (int)mdesc.size();
                    emitter->props.vec("radiance", P_COLOR, L.radiance, nullptr);
                    lights.push_back(L);
                    d.light = (int)lights.size() - 1;
                }
                mdesc.push_back(d);
                break;
            }
            case O_EMITTER: {
                dl_light_desc L;
                std::memset(&L, 0, sizeof(L));
                if (c->type == "point") {
                    L.type = DL_LIGHT_POINT;
                    L.mesh = -1;
                    c->props.vec("intensity", P_COLOR, L.radiance, nullptr);
                    c->props.vec("position", P_POINT, L.position, nullptr);
                } else if (c->type == "envmap") {
                    // src/tracer/emitter/envmap.cpp:13-19
                    std::string fn = c->props.s("filename");
                    if (!fn.empty() && fn[0] != '/') fn = it.dir + "/" + fn;
                    std::string ext = fn.size() >= 4 ? fn.substr(fn.size() - 4) : "";
                    for (char& ch : ext) ch = (char)std::tolower((unsigned char)ch);
                    if (ext != ".pfm")
                        throw Error(DL_ERR_UNSUPPORTED, "envmap \"" + fn + "\": only PFM images are read");
                    int w = 0, h = 0;
                    env_images.push_back(load_pfm(fn, w, h));
                    L.type = DL_LIGHT_ENVMAP;
                    L.mesh = -1;
                    L.env_rgb = env_images.back().data();
                    L.env_width = w;
                    L.env_height = h;
                    L.env_scale = c->props.f("scale", 1.0f);
                    L.env_visual = c->props.b("visual", true) ? 1 : 0;
                    const float zero[3] = {0.f, 0.f, 0.f};
                    scene->props.vec("bg_color", P_COLOR, L.env_background, zero);
                } else {
                    throw Error(DL_ERR_UNSUPPORTED, "emitter type \"" + c->type + "\" is not supported at scene level");
                }
                lights.push_back(L);
                break;
            }
            case O_CAMERA: {
                if (have_cam) throw Error(DL_ERR_PARSE, "There can only be one camera per scene!");
                have_cam = true;
                cam.width = c->props.i("width", 1280);
                cam.height = c->props.i("height", 720);
                if (c->type == "virtual") {  // virtual.cpp:16-30
                    cam.type = DL_CAMERA_VIRTUAL;
                    cam.fov = c->props.f("fov", 30.0f);
                    c->props.vec("eye", P_VECTOR, cam.eye, nullptr);
                    c->props.vec("lookat", P_VECTOR, cam.lookat, nullptr);
                    c->props.vec("up", P_VECTOR, cam.up, nullptr);
                } else if (c->type == "perspective") {  // perspective.cpp:21-38
                    cam.type = DL_CAMERA_PERSPECTIVE;
                    cam.fov = c->props.f("fov", 30.0f);
                    cam.near_clip = c->props.f("nearClip", 1e-4f);
                    cam.far_clip = c->props.f("farClip", 1e4f);
                    const M4 t = c->props.transform("toWorld");
                    for (int k = 0; k < 16; k++) cam.transform[k] = t.m[k / 4][k % 4];
                } else if (c->type == "opencv") {  // opencv.cpp:10-24
                    cam.type = DL_CAMERA_OPENCV;
                    cam.cx = c->props.f("cx");
                    cam.cy = c->props.f("cy");
                    cam.fx = c->props.f("fx");
                    cam.fy = c->props.f("fy");
                    if (!c->props.get("extrinsic", P_TRANSFORM)) c->props.missing("extrinsic");
                    const M4 t = c->props.transform("extrinsic");
                    for (int k = 0; k < 16; k++) cam.transform[k] = t.m[k / 4][k % 4];
                } else {
                    throw Error(DL_ERR_UNSUPPORTED, "camera type \"" + c->type + "\" is not supported");
                }
                for (Obj* ch : c->children) {
                    if (ch->kind != O_RFILTER) throw Error(DL_ERR_PARSE, "Camera::addChild: unsupported child");
                    if (ch->type == "gaussian") {
                        if (ch->props.f("radius", 2.0f) != 2.0f || ch->props.f("stddev", 0.5f) != 0.5f)
                            throw Error(DL_ERR_UNSUPPORTED, "only the default Gaussian filter (radius 2, stddev 0.5) is supported");
                        filter = DL_FILTER_GAUSSIAN;
                    } else if (ch->type == "box") {
                        filter = DL_FILTER_BOX;
                    } else {
                        throw Error(DL_ERR_UNSUPPORTED, "rfilter \"" + ch->type + "\" is not supported");
                    }
                }
                break;
            }
            case O_INTEGRATOR:
                if (have_integrator) throw Error(DL_ERR_PARSE, "There can only be one integrator per scene!");
                if (c->type == "normals") integrator_flags = DL_RENDER_NORMALS;  // normal.cpp:35
                else if (c->type != "path")
                    throw Error(DL_ERR_UNSUPPORTED, "integrator \"" + c->type + "\" is not supported");
                have_integrator = true;
                break;
            case O_SAMPLER:
                if (have_sampler) throw Error(DL_ERR_PARSE, "There can only be one sampler per scene!");
                if (c->type != "independent") throw Error(DL_ERR_UNSUPPORTED, "sampler \"" + c->type + "\" is not supported");
                have_sampler = true;
                spp = c->props.i("sampleCount", 1);
                break;
            case O_BSDF:
                break;  // pooled BSDF declared at scene level
            default:
                throw Error(DL_ERR_PARSE, "Scene::addChild: unsupported child");
        }
    }
    if (!have_integrator) throw Error(DL_ERR_PARSE, "No integrator was specified!");
    if (!have_cam) throw Error(DL_ERR_PARSE, "No camera was specified!");
    for (size_t i = 0; i < mdesc.size(); i++) {
        MeshData& m = meshdata[i];
        dl_mesh_desc& d = mdesc[i];
        d.positions = m.V.data();
        d.normals = m.N.empty() ? nullptr : m.N.data();
        d.texcoords = m.UV.empty() ? nullptr : m.UV.data();
        d.indices = m.F.data();
        d.num_vertices = (int64_t)(m.V.size() / 3);
        d.num_triangles = (int64_t)(m.F.size() / 3);
    }
    std::unique_ptr<dl_scene> S(new dl_scene());
    S->ctx = ctx;
    build_scene(S.get(), mdesc.data(), (int32_t)mdesc.size(), mats.data(), (int32_t)mats.size(), lights.data(),
                (int32_t)lights.size(), &cam);
    S->defaults.spp = spp;
    S->defaults.filter = filter;
    S->defaults.flags |= integrator_flags;
    *out = S.release();
    return DL_OK;
}

}  // namespace dl
