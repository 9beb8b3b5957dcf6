// JSON-case front end (see jsoncase.hpp).
#include "jsoncase.hpp"

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <set>
#include <sstream>
#include <stdexcept>

namespace dgtd {

// ============================================================================ JSON
const Json* Json::find(const std::string& key) const
{
    if (type != Object) return nullptr;
    for (const auto& kv : obj)
        if (kv.first == key) return &kv.second;
    return nullptr;
}

const Json& Json::at(const std::string& key) const
{
    const Json* j = find(key);
    if (!j) throw std::runtime_error("JSON: missing key '" + key + "'");
    return *j;
}

double Json::number() const
{
    if (type != Number) throw std::runtime_error("JSON: number expected");
    return num;
}

int Json::integer() const { return static_cast<int>(std::lround(number())); }

const std::string& Json::string() const
{
    if (type != String) throw std::runtime_error("JSON: string expected");
    return str;
}

std::vector<double> Json::numbers() const
{
    if (type != Array) throw std::runtime_error("JSON: array expected");
    std::vector<double> v;
    for (const auto& e : arr) v.push_back(e.number());
    return v;
}

namespace {

struct JsonParser {
    const std::string& s;
    size_t i = 0;
    explicit JsonParser(const std::string& t) : s(t) {}

    [[noreturn]] void fail(const std::string& what)
    {
        throw std::runtime_error("JSON parse error at offset " + std::to_string(i) + ": " + what);
    }
    void ws()
    {
        while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) ++i;
    }
    bool lit(const char* w)
    {
        size_t n = std::char_traits<char>::length(w);
        if (s.compare(i, n, w) == 0) { i += n; return true; }
        return false;
    }
    Json value()
    {
        ws();
        if (i >= s.size()) fail("unexpected end");
        Json j;
        const char c = s[i];
        if (c == '{') {
            j.type = Json::Object;
            ++i; ws();
            if (i < s.size() && s[i] == '}') { ++i; return j; }
            for (;;) {
                ws();
                if (i >= s.size() || s[i] != '"') fail("object key expected");
                std::string k = string();
                ws();
                if (i >= s.size() || s[i] != ':') fail("':' expected");
                ++i;
                j.obj.emplace_back(k, value());
                ws();
                if (i < s.size() && s[i] == ',') { ++i; continue; }
                if (i < s.size() && s[i] == '}') { ++i; return j; }
                fail("',' or '}' expected");
            }
        }
        if (c == '[') {
            j.type = Json::Array;
            ++i; ws();
            if (i < s.size() && s[i] == ']') { ++i; return j; }
            for (;;) {
                j.arr.push_back(value());
                ws();
                if (i < s.size() && s[i] == ',') { ++i; continue; }
                if (i < s.size() && s[i] == ']') { ++i; return j; }
                fail("',' or ']' expected");
            }
        }
        if (c == '"') { j.type = Json::String; j.str = string(); return j; }
        if (lit("true")) { j.type = Json::Bool; j.b = true; return j; }
        if (lit("false")) { j.type = Json::Bool; j.b = false; return j; }
        if (lit("null")) return j;
        // number
        const char* begin = s.c_str() + i;
        char* end = nullptr;
        const double v = std::strtod(begin, &end);
        if (end == begin) fail("value expected");
        i += static_cast<size_t>(end - begin);
        j.type = Json::Number;
        j.num = v;
        return j;
    }
    std::string string()
    {
        std::string out;
        ++i;   // opening quote
        while (i < s.size() && s[i] != '"') {
            if (s[i] == '\\') {
                if (++i >= s.size()) fail("bad escape");
                const char e = s[i];
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    if (i + 4 >= s.size()) fail("bad \\u escape");
                    const int cp = std::stoi(s.substr(i + 1, 4), nullptr, 16);
                    out += cp < 128 ? static_cast<char>(cp) : '?';
                    i += 4;
                    break;
                }
                default: out += e; break;
                }
                ++i;
            } else {
                out += s[i++];
            }
        }
        if (i >= s.size()) fail("unterminated string");
        ++i;
        return out;
    }
};

}  // namespace

Json parse_json(const std::string& text)
{
    JsonParser p(text);
    Json j = p.value();
    p.ws();
    if (p.i != text.size()) p.fail("trailing characters");
    return j;
}

// ============================================================================ gmsh 2.2
namespace {

// Second-order elements whose edge nodes sit within this distance of their straight edges' midpoints
// are straight (the reference's tolerance for its curved-element test).
constexpr double kCurvedTol = 1e-5;

// Largest distance from an edge node to the nearest midpoint of the element's straight edges
// (v: nc corner nodes, then nm edge nodes, indices into xyz). A second-order element with all its
// edge nodes on midpoints has an affine geometry map.
double edge_node_deviation(const std::vector<double>& xyz, const int32_t* v, int nc, int nm)
{
    double worst = 0.0;
    for (int k = 0; k < nm; ++k) {
        const double* xm = &xyz[3 * static_cast<size_t>(v[nc + k])];
        double best = INFINITY;
        for (int a = 0; a < nc; ++a)
            for (int b = a + 1; b < nc; ++b) {
                const double* xa = &xyz[3 * static_cast<size_t>(v[a])];
                const double* xb = &xyz[3 * static_cast<size_t>(v[b])];
                double d2 = 0.0;
                for (int r = 0; r < 3; ++r) {
                    const double d = xm[r] - 0.5 * (xa[r] + xb[r]);
                    d2 += d * d;
                }
                best = std::min(best, std::sqrt(d2));
            }
        worst = std::max(worst, best);
    }
    return worst;
}

}  // namespace

GmshMesh read_gmsh22(const std::string& path)
{
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open mesh file " + path);
    GmshMesh m;
    std::map<long, int32_t> node_index;
    std::string line;
    bool have_format = false, have_nodes = false;
    long curved = 0;          // second-order elements whose edge nodes are off the straight edges
    double max_dev = 0.0;
    bool second_order = false;
    while (std::getline(f, line)) {
        if (line.rfind("$MeshFormat", 0) == 0) {
            std::getline(f, line);
            std::istringstream is(line);
            double ver = 0; int ftype = 0, dsize = 0;
            is >> ver >> ftype >> dsize;
            if (std::floor(ver) != 2.0) throw std::runtime_error(path + ": gmsh format " + line + " (2.2 ASCII expected)");
            if (ftype != 0) throw std::runtime_error(path + ": binary gmsh files are not supported");
            have_format = true;
        } else if (line.rfind("$Nodes", 0) == 0) {
            std::getline(f, line);
            const long n = std::stol(line);
            m.xyz.reserve(3 * n);
            for (long k = 0; k < n; ++k) {
                std::getline(f, line);
                std::istringstream is(line);
                long id; double x, y, z;
                if (!(is >> id >> x >> y >> z)) throw std::runtime_error(path + ": bad node line: " + line);
                node_index[id] = static_cast<int32_t>(m.xyz.size() / 3);
                m.xyz.insert(m.xyz.end(), {x, y, z});
            }
            have_nodes = true;
        } else if (line.rfind("$Elements", 0) == 0) {
            if (!have_nodes) throw std::runtime_error(path + ": $Elements before $Nodes");
            std::getline(f, line);
            const long n = std::stol(line);
            for (long k = 0; k < n; ++k) {
                std::getline(f, line);
                std::istringstream is(line);
                long id; int type, ntags;
                if (!(is >> id >> type >> ntags)) throw std::runtime_error(path + ": bad element line: " + line);
                std::vector<long> tags(ntags);
                for (auto& t : tags) is >> t;
                const int phys = ntags > 0 ? static_cast<int>(tags[0]) : 0;
                auto nodes = [&](int cnt) {
                    std::vector<int32_t> v(cnt);
                    for (int q = 0; q < cnt; ++q) {
                        long nid;
                        if (!(is >> nid)) throw std::runtime_error(path + ": short element line: " + line);
                        auto it = node_index.find(nid);
                        if (it == node_index.end()) throw std::runtime_error(path + ": element references a missing node");
                        v[q] = it->second;
                    }
                    return v;
                };
                if (type == 4) {
                    auto v = nodes(4);
                    m.tets.insert(m.tets.end(), v.begin(), v.end());
                    m.tet_tag.push_back(phys);
                } else if (type == 2) {
                    auto v = nodes(3);
                    m.tris.insert(m.tris.end(), v.begin(), v.end());
                    m.tri_tag.push_back(phys);
                } else if (type == 11 || type == 9) {
                    // second-order tetrahedron (10 nodes) / triangle (6 nodes): corners first, then one
                    // node per edge. Straight when every edge node lies on the midpoint of one of the
                    // element's edges (the reference's curved-element test, HesthavenEvolution.cpp:207-241,
                    // with its absolute tolerance 1e-5); straight elements load as linear ones.
                    const int nc = (type == 11) ? 4 : 3;
                    auto v = nodes(type == 11 ? 10 : 6);
                    second_order = true;
                    const double dev = edge_node_deviation(m.xyz, v.data(), nc, static_cast<int>(v.size()) - nc);
                    if (dev > kCurvedTol && type == 11) {
                        // a curved tetrahedron keeps its edge nodes. gmsh orders them on the edges
                        // (0,1) (1,2) (0,2) (0,3) (2,3) (1,3); they are stored in the order
                        // (0,1) (0,2) (0,3) (1,2) (1,3) (2,3)
                        static const int slot_of[6] = {0, 3, 1, 2, 5, 4};
                        double pos[6][3];
                        for (int k = 0; k < 6; ++k)
                            for (int r = 0; r < 3; ++r) pos[slot_of[k]][r] = m.xyz[3 * static_cast<size_t>(v[4 + k]) + r];
                        m.curved_tets.push_back(static_cast<int32_t>(m.tet_tag.size()));
                        for (int q = 0; q < 6; ++q) m.curved_edges.insert(m.curved_edges.end(), pos[q], pos[q] + 3);
                        ++curved;
                        max_dev = std::max(max_dev, dev);
                    } else if (dev > kCurvedTol) {
                        ++curved;   // a curved triangle: its geometry comes from the tetrahedra
                    }
                    if (type == 11) {
                        m.tets.insert(m.tets.end(), v.begin(), v.begin() + 4);
                        m.tet_tag.push_back(phys);
                    } else {
                        m.tris.insert(m.tris.end(), v.begin(), v.begin() + 3);
                        m.tri_tag.push_back(phys);
                    }
                } else if (type == 29 || type == 20 || type == 21) {
                    throw std::runtime_error(path + ": third-order (curved) elements are not supported");
                } else if (type == 15 || type == 1 || type == 8 || type == 26 || type == 27 || type == 28) {
                    // points and lines: not part of a tetrahedral model
                } else {
                    throw std::runtime_error(path + ": unsupported gmsh element type " + std::to_string(type));
                }
            }
        }
    }
    if (!have_format) throw std::runtime_error(path + ": no $MeshFormat section");
    if (m.tets.empty()) throw std::runtime_error(path + ": no tetrahedra (only 3D meshes are supported)");
    if (second_order) {
        // keep only the corner nodes the (linear) elements use, in their original order
        std::vector<int32_t> remap(m.xyz.size() / 3, -1);
        for (int32_t v : m.tets) remap[v] = 0;
        for (int32_t v : m.tris) remap[v] = 0;
        std::vector<double> xyz;
        for (size_t k = 0; k < remap.size(); ++k)
            if (remap[k] == 0) {
                remap[k] = static_cast<int32_t>(xyz.size() / 3);
                xyz.insert(xyz.end(), m.xyz.begin() + 3 * k, m.xyz.begin() + 3 * k + 3);
            }
        for (auto& v : m.tets) v = remap[v];
        for (auto& v : m.tris) v = remap[v];
        m.xyz.swap(xyz);
    }
    (void)max_dev;
    return m;
}

void refine_uniform(GmshMesh& m)
{
    // curved parents: the position of each curved edge's node, and per tet its geometry
    static const int ea[6] = {0, 0, 0, 1, 1, 2}, eb[6] = {1, 2, 3, 2, 3, 3};
    std::map<std::pair<int32_t, int32_t>, std::array<double, 3>> curved_edge;
    std::vector<int64_t> curved_of(m.tet_tag.size(), -1);
    for (size_t q = 0; q < m.curved_tets.size(); ++q) {
        const int32_t e = m.curved_tets[q];
        curved_of[e] = static_cast<int64_t>(q);
        for (int k = 0; k < 6; ++k) {
            const int32_t a = m.tets[4 * e + ea[k]], b = m.tets[4 * e + eb[k]];
            const double* p = &m.curved_edges[18 * q + 3 * k];
            curved_edge[{std::min(a, b), std::max(a, b)}] = {p[0], p[1], p[2]};
        }
    }
    std::map<std::pair<int32_t, int32_t>, int32_t> mid;
    auto midpoint = [&](int32_t a, int32_t b) {
        auto key = std::make_pair(std::min(a, b), std::max(a, b));
        auto it = mid.find(key);
        if (it != mid.end()) return it->second;
        const int32_t id = static_cast<int32_t>(m.xyz.size() / 3);
        auto ce = curved_edge.find(key);
        // a curved edge's midpoint is its edge node (the quadratic edge at parameter 1/2)
        for (int d = 0; d < 3; ++d)
            m.xyz.push_back(ce != curved_edge.end() ? ce->second[d] : 0.5 * (m.xyz[3 * a + d] + m.xyz[3 * b + d]));
        mid[key] = id;
        return id;
    };
    std::vector<int32_t> tets, ttag, tris, rtag, ctets;
    std::vector<double> cedges;
    const size_t ne = m.tet_tag.size();
    for (size_t e = 0; e < ne; ++e) {
        const int32_t v0 = m.tets[4 * e], v1 = m.tets[4 * e + 1], v2 = m.tets[4 * e + 2], v3 = m.tets[4 * e + 3];
        const int32_t m01 = midpoint(v0, v1), m02 = midpoint(v0, v2), m03 = midpoint(v0, v3);
        const int32_t m12 = midpoint(v1, v2), m13 = midpoint(v1, v3), m23 = midpoint(v2, v3);
        const int32_t kids[8][4] = {{v0, m01, m02, m03}, {m01, v1, m12, m13}, {m02, m12, v2, m23}, {m03, m13, m23, v3},
                                    // the inner octahedron split along the m02-m13 diagonal
                                    {m01, m02, m03, m13}, {m01, m02, m12, m13}, {m02, m03, m13, m23},
                                    {m02, m12, m13, m23}};
        // the kids' vertices in the parent's barycentric coordinates (vertex k = e_k, midpoint of
        // (a, b) = (e_a + e_b) / 2), for curved parents
        static const int kid_pairs[8][4][2] = {
            {{0, 0}, {0, 1}, {0, 2}, {0, 3}}, {{0, 1}, {1, 1}, {1, 2}, {1, 3}},
            {{0, 2}, {1, 2}, {2, 2}, {2, 3}}, {{0, 3}, {1, 3}, {2, 3}, {3, 3}},
            {{0, 1}, {0, 2}, {0, 3}, {1, 3}}, {{0, 1}, {0, 2}, {1, 2}, {1, 3}},
            {{0, 2}, {0, 3}, {1, 3}, {2, 3}}, {{0, 2}, {1, 2}, {1, 3}, {2, 3}}};
        for (int kk = 0; kk < 8; ++kk) {
            const auto& k = kids[kk];
            tets.insert(tets.end(), k, k + 4);
            ttag.push_back(m.tet_tag[e]);
            if (curved_of[e] < 0) continue;
            // the kid's edge nodes: the parent's second-order map at the kid's edge midpoints
            const double* ed = &m.curved_edges[18 * curved_of[e]];
            double G[10][3];
            for (int q = 0; q < 4; ++q)
                for (int d = 0; d < 3; ++d) G[q][d] = m.xyz[3 * static_cast<size_t>(m.tets[4 * e + q]) + d];
            for (int q = 0; q < 6; ++q)
                for (int d = 0; d < 3; ++d) G[4 + q][d] = ed[3 * q + d];
            auto parent_map = [&](const double* l, double* x) {
                for (int d = 0; d < 3; ++d) {
                    double a = 0.0;
                    for (int q = 0; q < 4; ++q) a += l[q] * (2.0 * l[q] - 1.0) * G[q][d];
                    for (int q = 0; q < 6; ++q) a += 4.0 * l[ea[q]] * l[eb[q]] * G[4 + q][d];
                    x[d] = a;
                }
            };
            double lv[4][4];
            for (int q = 0; q < 4; ++q) {
                for (int r = 0; r < 4; ++r) lv[q][r] = 0.0;
                lv[q][kid_pairs[kk][q][0]] += 0.5;
                lv[q][kid_pairs[kk][q][1]] += 0.5;
            }
            double nodes[6][3], dev = 0.0;
            for (int q = 0; q < 6; ++q) {
                double l[4];
                for (int r = 0; r < 4; ++r) l[r] = 0.5 * (lv[ea[q]][r] + lv[eb[q]][r]);
                parent_map(l, nodes[q]);
                double d2 = 0.0;
                for (int d = 0; d < 3; ++d) {
                    const double mm = 0.5 * (m.xyz[3 * static_cast<size_t>(k[ea[q]]) + d] + m.xyz[3 * static_cast<size_t>(k[eb[q]]) + d]);
                    d2 += (nodes[q][d] - mm) * (nodes[q][d] - mm);
                }
                dev = std::max(dev, std::sqrt(d2));
            }
            if (dev > kCurvedTol) {
                ctets.push_back(static_cast<int32_t>(ttag.size() - 1));
                for (int q = 0; q < 6; ++q) cedges.insert(cedges.end(), nodes[q], nodes[q] + 3);
            }
        }
    }
    const size_t nt = m.tri_tag.size();
    for (size_t t = 0; t < nt; ++t) {
        const int32_t a = m.tris[3 * t], b = m.tris[3 * t + 1], c = m.tris[3 * t + 2];
        const int32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
        const int32_t kids[4][3] = {{a, ab, ca}, {ab, b, bc}, {ca, bc, c}, {ab, bc, ca}};
        for (const auto& k : kids) {
            tris.insert(tris.end(), k, k + 3);
            rtag.push_back(m.tri_tag[t]);
        }
    }
    m.tets.swap(tets);
    m.tet_tag.swap(ttag);
    m.tris.swap(tris);
    m.tri_tag.swap(rtag);
    m.curved_tets.swap(ctets);
    m.curved_edges.swap(cedges);
}

// ============================================================================ case
namespace {

constexpr double kSpeedOfLight = 299792458.0;           // m/s; modulation frequency Hz -> normalised units
// ohm; bulk conductivity S/m -> normalised units. The reference's value and expression,
// mu0_SI * c_SI with mu0_SI = 4 pi 1e-7 (src/math/PhysicalConstants.h, driver.cpp:963), so that
// a lossy case gets the same sigma to the last bit (the CODATA 376.730313668 differs by 5e-10).
constexpr double kFreeSpaceImpedance = 4.0 * M_PI * 1e-7 * kSpeedOfLight;
constexpr double kAutoDelaySigmas = 5.0;                 // automatic plane-wave delay (pulse this many sigmas upstream)

std::string dirname(const std::string& p)
{
    const size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

std::string stem(const std::string& p)
{
    size_t a = p.find_last_of('/');
    a = (a == std::string::npos) ? 0 : a + 1;
    size_t b = p.find_last_of('.');
    if (b == std::string::npos || b < a) b = p.size();
    return p.substr(a, b - a);
}

std::vector<int> int_list(const Json& j)
{
    std::vector<int> v;
    for (double x : j.numbers()) v.push_back(static_cast<int>(std::lround(x)));
    return v;
}

void vec3(const Json& j, double* out)
{
    auto v = j.numbers();
    out[0] = out[1] = out[2] = 0.0;
    for (size_t d = 0; d < v.size() && d < 3; ++d) out[d] = v[d];
}

double orient(const double* a, const double* b, const double* c, const double* d)
{
    const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    const double w[3] = {d[0] - a[0], d[1] - a[1], d[2] - a[2]};
    return u[0] * (v[1] * w[2] - v[2] * w[1]) - u[1] * (v[0] * w[2] - v[2] * w[0]) + u[2] * (v[0] * w[1] - v[1] * w[0]);
}

// The reference's case layout (validateCaseNamingStyle, driver.cpp:1487-1543): a folder named as
// the case holding <case>.json and <case>.msh, and model.filename = "<case>.msh" with no path.
void check_case_naming(const std::string& json_path, const Json& J, const std::string& dir, const std::string& name)
{
    const size_t dot = json_path.find_last_of('.');
    if (dot == std::string::npos || json_path.substr(dot) != ".json")
        throw std::runtime_error("input case file must be a .json file: " + json_path);
    const Json* model = J.find("model");
    const Json* fn = model ? model->find("filename") : nullptr;
    if (!fn || fn->type != Json::String)
        throw std::runtime_error("invalid JSON style in " + json_path + ": model.filename is required and must be a string");
    const std::string folder = dir.substr(dir.find_last_of('/') == std::string::npos ? 0 : dir.find_last_of('/') + 1);
    const std::string& filename = fn->string();
    const std::string expected = name + ".msh";
    const bool ok = folder == name && filename == expected && filename.find('/') == std::string::npos &&
                    std::ifstream(dir + "/" + expected).good();
    if (!ok)
        throw std::runtime_error("invalid case naming style for " + json_path +
                                 ": folder name, .json name, .msh name and model.filename must match (expected folder '" +
                                 name + "', model.filename '" + expected + "'; found folder '" + folder +
                                 "', model.filename '" + filename + "')");
}

}  // namespace

namespace {

// The largest frequency of the case's pulses (calculateMaximumSourceFrequency, driver.cpp:20-61):
// modulated Gaussians give carrier + c / (2 spread), else plain Gaussians c / (2 min spread),
// else 1 GHz.
double max_source_frequency(const Json& J)
{
    double min_spread = 1e300, max_freq = 0.0;
    bool gaussian = false, modulated = false;
    if (const Json* srcs = J.find("sources"))
        for (const Json& s : srcs->arr) {
            const Json* mag = s.find("magnitude");
            if (!mag) continue;
            if (mag->has("frequency") && mag->has("spread")) {
                const double f_edge = mag->at("frequency").number() + kSpeedOfLight / (2.0 * mag->at("spread").number());
                if (f_edge > max_freq) { max_freq = f_edge; modulated = true; }
            } else if (mag->has("type") && mag->at("type").type == Json::String && mag->at("type").string() == "gaussian" &&
                       mag->has("spread")) {
                const double sp = mag->at("spread").number();
                if (sp > 0.0 && sp < min_spread) { min_spread = sp; gaussian = true; }
            }
        }
    if (modulated) return max_freq;
    if (gaussian) return kSpeedOfLight / (2.0 * min_spread);
    return 1e9;
}

int sgbc_side(const Json& v)
{
    // assignBoundaryType (driver.cpp:1225-1239)
    const std::string& t = v.string();
    if (t == "PEC") return DGTD_BC_PEC;
    if (t == "PMC") return DGTD_BC_PMC;
    if (t == "SMA") return DGTD_BC_SMA;
    throw std::runtime_error("Incorrect sgbc_bdr_type defined in .json.");
}

// One "SGBC" boundary entry (driver.cpp:1298-1462): its layers with the automatic order and
// segment count, the optional sheets, and the sub-solver's recommended step
// (SGBCWrapper ctor, SolverExtension.cpp:509-541).
SgbcStackSpec parse_sgbc(const Json& bj, double max_freq)
{
    constexpr double mu0 = 4.0 * M_PI * 1e-7, eps0 = 8.8541878188e-12;
    SgbcStackSpec sp;
    std::vector<double> skin_depths;
    auto layer_of = [&](const Json& mj) {
        SgbcLayer L;
        L.eps = mj.has("relative_permittivity") ? mj.at("relative_permittivity").number() : 1.0;
        L.mu = mj.has("relative_permeability") ? mj.at("relative_permeability").number() : 1.0;
        if (!mj.has("bulk_conductivity"))
            throw std::runtime_error("SGBC layer defined without 'bulk_conductivity' parameter. Verify .json parameters.");
        const double sigma_si = mj.at("bulk_conductivity").number();
        L.sigma = sigma_si * kFreeSpaceImpedance;
        if (!mj.has("material_width")) throw std::runtime_error("SGBC layer must define 'material_width'.");
        L.width = mj.at("material_width").number();
        const double mu_si = L.mu * mu0, eps_si = L.eps * eps0;
        const double peclet = sigma_si > 0.0 ? sigma_si / (max_freq * eps_si) : 0.0;
        if (peclet > 100.0) L.order = 2;
        else if (peclet < 0.1 && sigma_si < 1e-3) L.order = 4;
        else L.order = 3;
        const double wavelength = 1.0 / (max_freq * std::sqrt(mu_si * eps_si));
        const int segs_per_wavelength = static_cast<int>(std::ceil(20.0 / L.order));
        const double dx_wave = wavelength / segs_per_wavelength;
        double dx_skin = std::numeric_limits<double>::max(), skin = 0.0;
        if (sigma_si > 0.0) {
            skin = 1.0 / std::sqrt(M_PI * max_freq * mu_si * sigma_si);
            dx_skin = skin / 2.0;
        }
        const int autoseg = static_cast<int>(std::ceil(L.width / std::min(dx_wave, dx_skin)));
        L.segments = std::clamp(autoseg, 4, 1000);
        if (mj.has("num_of_segments")) L.segments = mj.at("num_of_segments").integer();
        if (mj.has("order")) L.order = mj.at("order").integer();
        sp.layers.push_back(L);
        skin_depths.push_back((sigma_si > 0.0 && skin > 0.0) ? L.width / skin : 0.0);
    };
    if (const Json* ls = bj.find("layers")) {
        for (const Json& lj : ls->arr) layer_of(lj);
    } else if (const Json* mj = bj.find("material")) {
        layer_of(*mj);
    } else {
        throw std::runtime_error("SGBC boundary must define either 'material' or 'layers'. Verify .json parameters.");
    }
    bool left = false, right = false;
    auto sides = [&](const Json& src) {
        if (const Json* sb = src.find("sgbc_boundaries")) {
            if (const Json* l = sb->find("left")) { left = true; sp.left_bc = sgbc_side(*l); }
            if (const Json* r = sb->find("right")) { right = true; sp.right_bc = sgbc_side(*r); }
        }
    };
    sides(bj);
    if (!left && !right)
        if (const Json* mj = bj.find("material")) sides(*mj);
    // recommended sub-step: half the wave crossing time of a segment, relaxed by min(N^2, 50) for
    // layers N > 3 skin depths thick, minimum over layers (computed in seconds, as the reference)
    double rec = std::numeric_limits<double>::max();
    for (size_t i = 0; i < sp.layers.size(); ++i) {
        const SgbcLayer& L = sp.layers[i];
        const double dx = L.width / L.segments;
        double layer_dt = (dx * std::sqrt(L.eps * L.mu)) / kSpeedOfLight * 0.5;
        if (skin_depths[i] > 3.0) layer_dt *= std::min(skin_depths[i] * skin_depths[i], 50.0);
        rec = std::min(rec, layer_dt);
    }
    sp.sub_dt = rec * kSpeedOfLight;
    return sp;
}

}  // namespace

Case load_case(const std::string& json_path)
{
    std::ifstream jf(json_path);
    if (!jf) throw std::runtime_error("cannot open case file " + json_path);
    std::stringstream buf;
    buf << jf.rdbuf();
    const Json J = parse_json(buf.str());
    Case c;
    c.dir = dirname(json_path);
    c.name = stem(json_path);
    check_case_naming(json_path, J, c.dir, c.name);

    // ---- solver options (driver.cpp:644-705)
    if (const Json* so = J.find("solver_options")) {
        if (const Json* v = so->find("upwind_alpha")) c.alpha = v->number();
        if (const Json* v = so->find("time_step")) c.dt = v->number();
        if (const Json* v = so->find("final_time")) c.final_time = v->number();
        if (const Json* v = so->find("cfl")) c.cfl = v->number();
        if (const Json* v = so->find("order")) c.order = v->integer();
        if (const Json* v = so->find("evolution_operator")) {
            // the reference's three names (driver.cpp:679-691); all run on this library's operator
            c.evolution_operator = v->string();
            if (c.evolution_operator != "maxwell" && c.evolution_operator != "global" &&
                c.evolution_operator != "hesthaven")
                throw std::runtime_error("wrong type of evolution operator '" + c.evolution_operator +
                                         "': choose 'maxwell', 'global' or 'hesthaven'");
        }
        if (const Json* v = so->find("basis_type")) {
            // MFEM's BasisType numbering (SolverOptions.h:74-77; 0 Gauss-Legendre, 1 Gauss-Lobatto,
            // 2 positive/Bernstein, ...). The operator runs on the Gauss-Lobatto node set; a
            // Gauss-Legendre case is the same polynomial space, whose state the runner maps to and
            // from that node set (the reference's integration rules are exact on straight elements,
            // so both bases give the same semi-discrete system)
            const int bt = v->integer();
            if (bt != 0 && bt != 1)
                throw std::runtime_error("basis_type " + std::to_string(bt) +
                                         " is not supported (Gauss-Legendre, 0, and Gauss-Lobatto, 1, are)");
            c.basis_type = bt;
        }
        if (const Json* v = so->find("ode_type")) {
            if (v->type == Json::String) {   // this library's names (LSERK4 has no number in the reference)
                const std::string& o = v->string();
                if (o == "RK4" || o == "rk4") c.integrator = DGTD_RK4;
                else if (o == "LSERK4" || o == "lserk4") c.integrator = DGTD_LSERK4;
                else throw std::runtime_error("ode_type '" + o + "' is not supported (RK4, LSERK4)");
            } else {
                // the reference's numbering (SolverOptions.h:8-16, Solver.cpp:41-77): 0 = RK4,
                // 1-6 the implicit solvers (BackwardEuler, Trapezoidal, ImplicitMidpoint, SDIRK33,
                // SDIRK23, SDIRK34)
                const int o = v->integer();
                if (o == 0) c.integrator = DGTD_RK4;
                else if (o >= 1 && o <= 6)
                    throw std::runtime_error("implicit ode_type " + std::to_string(o) +
                                             " is not supported (the explicit RK4, ode_type 0, is)");
                else
                    throw std::runtime_error("wrong ode type defined in json (ode_type " + std::to_string(o) + ")");
            }
        }
    }
    if (c.order < 1 || c.order > 6) throw std::runtime_error("order must be in [1, 6]");

    // ---- mesh (driver.cpp:1063-1188, 1242-1479)
    const Json& model = J.at("model");
    GmshMesh g = read_gmsh22(c.dir + "/" + model.at("filename").string());
    if (const Json* r = model.find("refinement"))
        for (int k = 0; k < r->integer(); ++k) refine_uniform(g);
    const int64_t K = static_cast<int64_t>(g.tet_tag.size());
    c.vertices = g.xyz;
    c.elements = g.tets;
    std::vector<int64_t> curved_of(K, -1);
    for (size_t q = 0; q < g.curved_tets.size(); ++q) curved_of[g.curved_tets[q]] = static_cast<int64_t>(q);
    for (int64_t e = 0; e < K; ++e) {
        int32_t* v = &c.elements[4 * e];
        const double* X = c.vertices.data();
        const bool flip = orient(X + 3 * v[0], X + 3 * v[1], X + 3 * v[2], X + 3 * v[3]) < 0.0;
        if (flip) std::swap(v[2], v[3]);
        if (curved_of[e] >= 0) {
            // corners in the (possibly swapped) vertex order, then the edges; swapping corners 2 and
            // 3 exchanges the edges (0,2) <-> (0,3) and (1,2) <-> (1,3)
            static const int keep[6] = {0, 1, 2, 3, 4, 5}, swapped[6] = {0, 2, 1, 4, 3, 5};
            const double* ed = &g.curved_edges[18 * curved_of[e]];
            c.curved_elems.push_back(static_cast<int32_t>(e));
            for (int k = 0; k < 4; ++k) c.curved_nodes.insert(c.curved_nodes.end(), X + 3 * v[k], X + 3 * v[k] + 3);
            for (int q = 0; q < 6; ++q) {
                const int src = flip ? swapped[q] : keep[q];
                c.curved_nodes.insert(c.curved_nodes.end(), ed + 3 * src, ed + 3 * src + 3);
            }
        }
    }

    // ---- materials by volume tag (driver.cpp:946-982): the first entry of a tag wins, a tag the
    // mesh does not have is an error, and no materials at all means vacuum on attribute 1
    // (Model.cpp:61-66)
    std::map<int, std::array<double, 3>> mat;
    const std::set<int> mesh_tags(g.tet_tag.begin(), g.tet_tag.end());
    for (const Json& mj : model.at("materials").arr) {
        std::array<double, 3> em = {1.0, 1.0, 0.0};
        if (const Json* v = mj.find("relative_permittivity")) em[0] = v->number();
        if (const Json* v = mj.find("relative_permeability")) em[1] = v->number();
        if (const Json* v = mj.find("bulk_conductivity")) em[2] = v->number() * kFreeSpaceImpedance;
        for (int t : int_list(mj.at("tags"))) {
            if (!mesh_tags.count(t))
                throw std::runtime_error("there is no attribute " + std::to_string(t) +
                                         " defined in the mesh, but it is defined in the JSON");
            mat.emplace(t, em);
        }
    }
    if (mat.empty()) mat.emplace(1, std::array<double, 3>{1.0, 1.0, 0.0});
    c.eps.resize(K); c.mu.resize(K); c.sigma.resize(K);
    for (int64_t e = 0; e < K; ++e) {
        auto it = mat.find(g.tet_tag[e]);
        if (it == mat.end())
            throw std::runtime_error("element attribute " + std::to_string(g.tet_tag[e]) + " has no material in the case");
        c.eps[e] = it->second[0]; c.mu[e] = it->second[1]; c.sigma[e] = it->second[2];
    }

    // ---- face -> elements map of the tagged triangles
    using Key = std::array<int32_t, 3>;
    auto key_of = [](int32_t a, int32_t b, int32_t d) { Key k{a, b, d}; std::sort(k.begin(), k.end()); return k; };
    std::map<Key, std::vector<int64_t>> face_elems;
    for (size_t t = 0; t < g.tri_tag.size(); ++t) face_elems[key_of(g.tris[3 * t], g.tris[3 * t + 1], g.tris[3 * t + 2])];
    for (int64_t e = 0; e < K; ++e)
        for (int f = 0; f < 4; ++f) {
            int32_t v[3]; int q = 0;
            for (int k = 0; k < 4; ++k) if (k != f) v[q++] = c.elements[4 * e + k];
            auto it = face_elems.find(key_of(v[0], v[1], v[2]));
            if (it != face_elems.end()) it->second.push_back(e);
        }
    auto barycentre = [&](int64_t e, double* out) {
        out[0] = out[1] = out[2] = 0.0;
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) out[d] += 0.25 * c.vertices[3 * c.elements[4 * e + k] + d];
    };

    // ---- plane waves (driver.cpp:565-609) and their TF/SF surfaces (SubMesher.cpp:677-775)
    std::set<int> tfsf_tags;
    if (const Json* srcs = J.find("sources")) {
        for (const Json& s : srcs->arr) {
            const std::string& type = s.at("type").string();
            if (type == "planewave") {
                const Json& mag = s.at("magnitude");
                dgtd_planewave w{};
                vec3(s.at("propagation"), w.propagation);
                vec3(s.at("polarization"), w.polarization);
                w.spread = mag.at("spread").number();
                const double kn = std::sqrt(w.propagation[0] * w.propagation[0] + w.propagation[1] * w.propagation[1] +
                                            w.propagation[2] * w.propagation[2]);
                if (!(kn > 0.0)) throw std::runtime_error("plane wave with zero propagation");
                const double kh[3] = {w.propagation[0] / kn, w.propagation[1] / kn, w.propagation[2] / kn};
                std::vector<int> tags = s.has("tags") ? int_list(s.at("tags")) : std::vector<int>();
                if (const Json* m = mag.find("mean")) {
                    // a position (the reference reads it with assemble3DVector, driver.cpp:346-353,
                    // 574-575, which fails on a plain number as well)
                    if (m->type != Json::Array)
                        throw std::runtime_error("plane wave magnitude.mean must be a 3-vector (a position on "
                                                 "the propagation axis), not a number");
                    double mv[3];
                    vec3(*m, mv);
                    w.mean = mv[0] * kh[0] + mv[1] * kh[1] + mv[2] * kh[2];
                } else {
                    // automatic delay: the pulse peak kAutoDelaySigmas sqrt(2) spreads upstream of
                    // the earliest TF/SF surface element centroid (driver.cpp:455-472, 576-589)
                    double min_phase = 1e300;
                    for (size_t t = 0; t < g.tri_tag.size(); ++t) {
                        if (std::find(tags.begin(), tags.end(), g.tri_tag[t]) == tags.end()) continue;
                        double ph = 0.0;
                        for (int d = 0; d < 3; ++d) {
                            double x = 0.0;
                            for (int k = 0; k < 3; ++k) x += g.xyz[3 * g.tris[3 * t + k] + d] / 3.0;
                            ph += x * kh[d];
                        }
                        min_phase = std::min(min_phase, ph);
                    }
                    if (min_phase == 1e300) min_phase = 0.0;
                    w.mean = min_phase - kAutoDelaySigmas * w.spread * std::sqrt(2.0);
                }
                if (const Json* fr = mag.find("frequency")) w.frequency = fr->number() / kSpeedOfLight;
                w.batch = 0;
                c.waves.push_back(w);
                for (int t : tags) tfsf_tags.insert(t);
            } else if (type == "initial") {
                CaseInitialField f;
                const std::string& ft = s.at("field_type").string();
                if (ft == "electric") f.field = 0;
                else if (ft == "magnetic") f.field = 1;
                else throw std::runtime_error("initial field_type must be electric or magnetic");
                vec3(s.at("polarization"), f.pol);
                const Json& mag = s.at("magnitude");
                const std::string& mt = mag.at("type").string();
                if (mt == "gaussian") {
                    f.kind = 0;
                    f.spread = mag.at("spread").number();
                    vec3(s.at("center"), f.center);
                    f.dimension = s.has("dimension") ? s.at("dimension").integer() : 1;
                    if (f.dimension < 1 || f.dimension > 3) throw std::runtime_error("gaussian dimension must be 1..3");
                } else if (mt == "resonant") {
                    f.kind = 1;
                    f.modes = int_list(mag.at("modes"));
                } else if (mt == "besselj6_2D") {   // driver.cpp:552-557, Function.h:170-193
                    f.kind = 2;
                } else if (mt == "besselj6_3D") {   // driver.cpp:558-563, Function.h:195-226
                    f.kind = 3;
                } else {
                    throw std::runtime_error("initial field magnitude '" + mt +
                                             "' is not supported (gaussian, resonant, besselj6_2D, besselj6_3D)");
                }
                c.initial.push_back(f);
            } else {
                throw std::runtime_error("source type '" + type + "' is not supported (initial, planewave)");
            }
        }
    }
    if (!tfsf_tags.empty()) {
        // total-field side: the element whose barycentre is closer to the centroid of the
        // TF/SF surface vertices; the winding normal of each face points into it
        double cen[3] = {0, 0, 0};
        std::set<int32_t> verts;
        for (size_t t = 0; t < g.tri_tag.size(); ++t)
            if (tfsf_tags.count(g.tri_tag[t]))
                for (int k = 0; k < 3; ++k) verts.insert(g.tris[3 * t + k]);
        for (int32_t v : verts)
            for (int d = 0; d < 3; ++d) cen[d] += g.xyz[3 * v + d] / static_cast<double>(verts.size());
        for (size_t t = 0; t < g.tri_tag.size(); ++t) {
            if (!tfsf_tags.count(g.tri_tag[t])) continue;
            int32_t a = g.tris[3 * t], b = g.tris[3 * t + 1], d = g.tris[3 * t + 2];
            const auto& el = face_elems[key_of(a, b, d)];
            if (el.size() != 2) throw std::runtime_error("TF/SF surface faces must lie between two elements");
            double b0[3], b1[3];
            barycentre(el[0], b0);
            barycentre(el[1], b1);
            double d0 = 0, d1 = 0;
            for (int q = 0; q < 3; ++q) { d0 += (b0[q] - cen[q]) * (b0[q] - cen[q]); d1 += (b1[q] - cen[q]) * (b1[q] - cen[q]); }
            const double* tf = d0 < d1 ? b0 : b1;
            const double* A = &c.vertices[3 * a];
            const double* B = &c.vertices[3 * b];
            const double* D = &c.vertices[3 * d];
            if (orient(A, B, D, tf) < 0.0) std::swap(b, d);
            c.tfsf_faces.insert(c.tfsf_faces.end(), {a, b, d});
        }
    }

    // ---- boundaries by surface tag (driver.cpp:985-1049). As in the reference: every entry needs
    // non-empty tags and a type; the first entry of a tag wins; a tag is an interior boundary as a
    // whole when any of its faces lies between two elements, and then only its interior faces get
    // the condition (the reference applies interior-boundary tags through interior face
    // integrators only, so that tag's faces on the domain boundary keep no condition: open).
    std::map<int, int> bc_of_tag;
    std::map<int, int> sgbc_of_tag;   // tag -> stack
    const double max_freq = max_source_frequency(J);
    if (const Json* bs = model.find("boundaries")) {
        for (size_t b = 0; b < bs->arr.size(); ++b) {
            const Json& bj = bs->arr[b];
            const Json* tj = bj.find("tags");
            if (!tj) throw std::runtime_error("boundary " + std::to_string(b) + " does not have defined 'tags'");
            const std::vector<int> tags = int_list(*tj);
            if (tags.empty()) throw std::runtime_error("boundary " + std::to_string(b) + " 'tags' are empty");
            const Json* ty = bj.find("type");
            if (!ty) throw std::runtime_error("boundary " + std::to_string(b) + " does not have a defined 'type'");
            const std::string& type = ty->string();
            int code;
            if (type == "PEC") code = DGTD_BC_PEC;
            else if (type == "PMC") code = DGTD_BC_PMC;
            else if (type == "SMA") code = DGTD_BC_SMA;
            else if (type == "SGBC") code = DGTD_BC_SGBC;
            else throw std::runtime_error("boundary type '" + type + "' is not supported (PEC, PMC, SMA, SGBC)");
            if (code == DGTD_BC_SGBC) {
                const int idx = static_cast<int>(c.sgbc_stacks.size());
                c.sgbc_stacks.push_back(parse_sgbc(bj, max_freq));
                for (int t : tags) sgbc_of_tag.emplace(t, idx);
            }
            for (int t : tags) bc_of_tag.emplace(t, code);
        }
    }
    std::vector<int> tri_nelem(g.tri_tag.size());
    std::set<int> interior_tags;
    for (size_t t = 0; t < g.tri_tag.size(); ++t) {
        if (!bc_of_tag.count(g.tri_tag[t])) continue;
        const auto& el = face_elems[key_of(g.tris[3 * t], g.tris[3 * t + 1], g.tris[3 * t + 2])];
        if (el.size() != 1 && el.size() != 2)
            throw std::runtime_error("tagged surface triangle is not a face of the tetrahedral mesh");
        tri_nelem[t] = static_cast<int>(el.size());
        if (el.size() == 2) interior_tags.insert(g.tri_tag[t]);
    }
    for (size_t t = 0; t < g.tri_tag.size(); ++t) {
        const int tag = g.tri_tag[t];
        auto it = bc_of_tag.find(tag);
        if (it == bc_of_tag.end()) continue;
        const int32_t a = g.tris[3 * t], b = g.tris[3 * t + 1], d = g.tris[3 * t + 2];
        if (interior_tags.count(tag)) {
            if (tri_nelem[t] == 2) {
                c.int_faces.insert(c.int_faces.end(), {a, b, d});
                c.int_codes.push_back(it->second);
                if (it->second == DGTD_BC_SGBC) c.sgbc_face_stack.push_back(sgbc_of_tag.at(tag));
            }
        } else if (it->second == DGTD_BC_SGBC) {
            // an SGBC tag on the domain boundary: the reference's operator gives these faces the
            // boundary coefficients {1, 1} (SMA's) scaled by alpha (DGOperatorFactory.h:21-35,
            // 483-497), and its source-face operator, assembled on interior faces, injects nothing
            if (c.alpha != 1.0)
                throw std::runtime_error("SGBC on the domain boundary (tag " + std::to_string(tag) +
                                         ") is supported with upwind_alpha 1 only (SMA coefficients scaled by alpha)");
            c.bdr_faces.insert(c.bdr_faces.end(), {a, b, d});
            c.bdr_codes.push_back(DGTD_BC_SMA);
        } else {
            c.bdr_faces.insert(c.bdr_faces.end(), {a, b, d});
            c.bdr_codes.push_back(it->second);
        }
    }

    // ---- probes (driver.cpp:707-868): "steps" is the interval; "saves" asks for that many samples
    // over the run, turned into an interval with the run's dt (placeholder 1 while dt is automatic)
    auto saves_of = [](const Json& pj) { return pj.has("saves") ? pj.at("saves").integer() : 0; };
    auto interval_of = [&](const Json& pj) {
        if (const Json* st = pj.find("steps")) return std::max(1, st->integer());
        if (pj.has("saves")) return c.dt > 0.0 ? probe_interval(saves_of(pj), 1, c.final_time, c.dt) : 1;
        return 1;
    };
    if (const Json* pr = J.find("probes")) {
        if (const Json* pts = pr->find("point"))
            for (const Json& pj : pts->arr) {
                double x[3];
                vec3(pj.at("position"), x);
                c.point_pos.insert(c.point_pos.end(), {x[0], x[1], x[2]});
                c.point_interval.push_back(interval_of(pj));
                c.point_saves.push_back(saves_of(pj));
            }
        for (const char* kind : {"rcssurface", "farfield"})
            if (const Json* surf = pr->find(kind))
                for (const Json& sj : surf->arr) {
                    CaseSurface s;
                    s.name = sj.has("name") ? sj.at("name").string() : std::string(kind);
                    s.interval = interval_of(sj);
                    if (sj.has("tags")) s.tags = int_list(sj.at("tags"));
                    // orient each face away from the centroid of the surface's vertices
                    double cen[3] = {0, 0, 0};
                    std::set<int32_t> verts;
                    for (size_t t = 0; t < g.tri_tag.size(); ++t)
                        if (std::find(s.tags.begin(), s.tags.end(), g.tri_tag[t]) != s.tags.end())
                            for (int k = 0; k < 3; ++k) verts.insert(g.tris[3 * t + k]);
                    for (int32_t v : verts)
                        for (int d = 0; d < 3; ++d) cen[d] += g.xyz[3 * v + d] / static_cast<double>(verts.size());
                    for (size_t t = 0; t < g.tri_tag.size(); ++t) {
                        if (std::find(s.tags.begin(), s.tags.end(), g.tri_tag[t]) == s.tags.end()) continue;
                        int32_t a = g.tris[3 * t], b = g.tris[3 * t + 1], d = g.tris[3 * t + 2];
                        if (orient(&c.vertices[3 * a], &c.vertices[3 * b], &c.vertices[3 * d], cen) > 0.0) std::swap(b, d);
                        s.faces.insert(s.faces.end(), {a, b, d});
                    }
                    c.surfaces.push_back(s);
                }
    }
    if (!c.sgbc_face_stack.empty() && c.evolution_operator != "global")
        throw std::runtime_error("thin-layer (SGBC) boundaries run with evolution_operator 'global' only "
                                 "(the reference couples them in GlobalEvolution)");
    if (c.basis_type == 0) {
        // The change of basis is exact where the operator is basis-free: straight elements
        // (curved ones integrate non-polynomial terms), no source sampled at the nodes (a plane
        // wave is interpolated on the case's node set), no face-node sub-solvers (SGBC), and not
        // the Hesthaven evolution (built on face nodes)
        if (!c.curved_elems.empty())
            throw std::runtime_error("basis_type 0 (Gauss-Legendre) with curved elements is not supported");
        if (!c.waves.empty())
            throw std::runtime_error("basis_type 0 (Gauss-Legendre) with plane-wave sources is not supported");
        if (!c.sgbc_face_stack.empty())
            throw std::runtime_error("basis_type 0 (Gauss-Legendre) with SGBC boundaries is not supported");
        if (c.evolution_operator == "hesthaven")
            throw std::runtime_error("basis_type 0 (Gauss-Legendre) with the hesthaven evolution is not supported");
    }
    return c;
}

int probe_interval(int saves, int steps_interval, double final_time, double dt)
{
    if (saves <= 0 || !(dt > 0.0)) return steps_interval;
    const int total = static_cast<int>(std::ceil(final_time / dt));
    return std::max(1, total / saves);
}

namespace {

// Spherical Bessel function j_l(x): below x = l + 2 the power series
// x^l sum_k (-x^2 / 2)^k / (k! (2l + 2k + 1)!!), above it the upward recurrence
// j_(k+1) = (2k + 1) / x j_k - j_(k-1) from j_0 = sin x / x and j_1 = sin x / x^2 - cos x / x.
double sph_bessel_j(int l, double x)
{
    if (x == 0.0) return l == 0 ? 1.0 : 0.0;
    if (x < l + 2.0) {
        double dfact = 1.0;
        for (int k = 1; k <= 2 * l + 1; k += 2) dfact *= k;
        double term = std::pow(x, l) / dfact, sum = term;
        for (int k = 1; k < 80; ++k) {
            term *= -x * x / (2.0 * k * (2.0 * l + 2.0 * k + 1.0));
            sum += term;
            if (std::fabs(term) < 1e-18 * std::fabs(sum)) break;
        }
        return sum;
    }
    double j0 = std::sin(x) / x, j1 = std::sin(x) / (x * x) - std::cos(x) / x;
    if (l == 0) return j0;
    for (int k = 1; k < l; ++k) {
        const double j2 = (2.0 * k + 1.0) / x * j1 - j0;
        j0 = j1;
        j1 = j2;
    }
    return j1;
}

// The reference's Bessel cavity fields at t = 0 (alpha6 = 13.589290170541217, the second zero of
// J_6): 2D: J_6(alpha6 rho) cos(6 phi); 3D: j_6(alpha6 r) Y_66(theta, phi) with the normalised
// associated Legendre function sqrt(13 / (4 pi) / 12!) 11!! sin^6(theta) (Condon-Shortley sign
// (-1)^6 = 1).
constexpr double kAlpha6 = 13.589290170541217;

double besselj6_2d(const double* p)
{
    return ::jn(6, kAlpha6 * std::sqrt(p[0] * p[0] + p[1] * p[1])) * std::cos(6.0 * std::atan2(p[1], p[0]));
}

double besselj6_3d(const double* p)
{
    const double r = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    if (r == 0.0) return 0.0;
    const double c = p[2] / r, s2 = 1.0 - c * c;
    const double P66 = std::sqrt(13.0 / (4.0 * M_PI) / 479001600.0) * 10395.0 * s2 * s2 * s2;
    return sph_bessel_j(6, kAlpha6 * r) * P66 * std::cos(6.0 * std::atan2(p[1], p[0]));
}

}  // namespace

std::vector<double> case_initial_state(const Case& c, const double* xyz, int64_t n)
{
    std::vector<double> u(6 * static_cast<size_t>(n), 0.0);
    for (const auto& f : c.initial) {
        for (int64_t i = 0; i < n; ++i) {
            const double p[3] = {xyz[i], xyz[n + i], xyz[2 * n + i]};
            double v;
            if (f.kind == 0) {
                double r2 = 0.0;
                for (int d = 0; d < f.dimension; ++d) r2 += (p[d] - f.center[d]) * (p[d] - f.center[d]);
                v = std::exp(-r2 / (2.0 * f.spread * f.spread));
            } else if (f.kind == 1) {
                v = 1.0;
                for (size_t d = 0; d < f.modes.size() && d < 3; ++d) v *= std::sin(f.modes[d] * M_PI * p[d]);
            } else if (f.kind == 2) {
                v = besselj6_2d(p);
            } else {
                v = besselj6_3d(p);
            }
            for (int k = 0; k < 3; ++k) u[(3 * f.field + k) * static_cast<size_t>(n) + i] += v * f.pol[k];
        }
    }
    return u;
}

}  // namespace dgtd
