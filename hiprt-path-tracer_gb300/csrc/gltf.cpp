// glTF 2.0 scene ingestion for the render path: the reference's sample scenes (data/GLTFs/*.gltf)
// become a gbpt_scene_desc (world-space triangles, per-triangle material indices, principled
// materials) and a camera, without ASSIMP.
//
// The reference reads scenes through ASSIMP (SceneParser::parse_scene_file,
// src/Scene/SceneParser.cpp:21-226, post-processing aiProcess_PreTransformVertices |
// aiProcess_Triangulate) and maps each aiMaterial with read_material_properties
// (src/Scene/SceneParser.cpp:391-438) followed by CPUMaterial::make_safe
// (src/HostDeviceCommon/Material/MaterialCPU.h:156-207). This file reads the glTF JSON and its
// buffers directly:
//   * the default scene's node tree is walked depth first and every mesh instance is transformed
//     to world space (what PreTransformVertices does), winding flipped under mirroring transforms
//     as the glTF specification asks;
//   * triangle lists, strips and fans become triangles (what Triangulate does for glTF);
//   * the material keys the reference reads are taken from the glTF fields ASSIMP's glTF 2 importer
//     fills them from, with the same "only when present" behaviour for the extension keys.
// Everything here is host code: parsing is not on the render hot path.

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "handles.h"
#include "../../include/gbpt_render.h"

namespace {

struct GltfError
{
    gbpt_status status;
    std::string msg;
};

[[noreturn]] void fail(const std::string& msg, gbpt_status s = GBPT_ERROR_INVALID_ARG)
{
    throw GltfError{s, msg};
}

// ---- a small JSON reader (RFC 8259 values; numbers as double) ----

struct Json
{
    enum Kind : uint8_t { Null, Bool, Number, String, Array, Object };
    Kind kind = Null;
    bool boolean = false;
    double number = 0.0;
    std::string text;
    std::vector<Json> items;                            // Array
    std::vector<std::pair<std::string, Json>> members;  // Object, in file order

    const Json* find(const char* key) const
    {
        if (kind != Object)
            return nullptr;
        for (const auto& m : members)
            if (m.first == key)
                return &m.second;
        return nullptr;
    }
    bool has(const char* key) const { return find(key) != nullptr; }
};

class JsonReader
{
public:
    JsonReader(const char* begin, const char* end) : p_(begin), end_(end), begin_(begin) {}

    Json parse_document()
    {
        Json v;
        skip_space();
        parse_value(v, 0);
        skip_space();
        if (p_ != end_)
            error("trailing characters after the JSON document");
        return v;
    }

private:
    static constexpr int kMaxDepth = 256;
    const char* p_;
    const char* end_;
    const char* begin_;

    [[noreturn]] void error(const char* what) const
    {
        fail(std::string("glTF JSON: ") + what + " at byte " + std::to_string(p_ - begin_));
    }

    void skip_space()
    {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r'))
            ++p_;
    }

    bool take(char c)
    {
        if (p_ < end_ && *p_ == c) {
            ++p_;
            return true;
        }
        return false;
    }

    void expect_word(const char* w)
    {
        for (; *w; ++w, ++p_)
            if (p_ >= end_ || *p_ != *w)
                error("invalid literal");
    }

    void parse_value(Json& v, int depth)
    {
        if (depth > kMaxDepth)
            error("nesting too deep");
        if (p_ >= end_)
            error("unexpected end of input");
        const char c = *p_;
        if (c == '{') {
            ++p_;
            v.kind = Json::Object;
            skip_space();
            if (take('}'))
                return;
            for (;;) {
                skip_space();
                if (p_ >= end_ || *p_ != '"')
                    error("expected an object key");
                std::string key;
                parse_string(key);
                skip_space();
                if (!take(':'))
                    error("expected ':'");
                skip_space();
                v.members.emplace_back(std::move(key), Json());
                parse_value(v.members.back().second, depth + 1);
                skip_space();
                if (take(','))
                    continue;
                if (take('}'))
                    return;
                error("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p_;
            v.kind = Json::Array;
            skip_space();
            if (take(']'))
                return;
            for (;;) {
                skip_space();
                v.items.emplace_back();
                parse_value(v.items.back(), depth + 1);
                skip_space();
                if (take(','))
                    continue;
                if (take(']'))
                    return;
                error("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Json::String;
            parse_string(v.text);
            return;
        }
        if (c == 't') {
            expect_word("true");
            v.kind = Json::Bool;
            v.boolean = true;
            return;
        }
        if (c == 'f') {
            expect_word("false");
            v.kind = Json::Bool;
            return;
        }
        if (c == 'n') {
            expect_word("null");
            return;
        }
        parse_number(v);
    }

    static bool digit(char c) { return c >= '0' && c <= '9'; }

    void parse_number(Json& v)
    {
        // Checks the JSON number grammar, then converts the checked span with strtod (the C
        // library's correctly rounded conversion; the span holds no locale-dependent characters
        // other than '.', which the "C" numeric locale every process starts in reads).
        const char* s = p_;
        take('-');
        if (p_ < end_ && *p_ == '0')
            ++p_;
        else if (p_ < end_ && digit(*p_) && *p_ != '0')
            while (p_ < end_ && digit(*p_))
                ++p_;
        else
            error("invalid number");
        if (take('.')) {
            if (p_ >= end_ || !digit(*p_))
                error("invalid number");
            while (p_ < end_ && digit(*p_))
                ++p_;
        }
        if (p_ < end_ && (*p_ == 'e' || *p_ == 'E')) {
            ++p_;
            if (!take('+'))
                take('-');
            if (p_ >= end_ || !digit(*p_))
                error("invalid number");
            while (p_ < end_ && digit(*p_))
                ++p_;
        }
        const std::string span(s, p_);
        v.kind = Json::Number;
        v.number = std::strtod(span.c_str(), nullptr);
    }

    unsigned hex4()
    {
        unsigned u = 0;
        for (int i = 0; i < 4; ++i, ++p_) {
            if (p_ >= end_)
                error("truncated \\u escape");
            const char c = *p_;
            u <<= 4;
            if (c >= '0' && c <= '9')
                u |= unsigned(c - '0');
            else if (c >= 'a' && c <= 'f')
                u |= unsigned(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F')
                u |= unsigned(c - 'A' + 10);
            else
                error("invalid \\u escape");
        }
        return u;
    }

    static void put_utf8(std::string& out, unsigned cp)
    {
        if (cp < 0x80) {
            out += char(cp);
        } else if (cp < 0x800) {
            out += char(0xC0 | (cp >> 6));
            out += char(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += char(0xE0 | (cp >> 12));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        } else {
            out += char(0xF0 | (cp >> 18));
            out += char(0x80 | ((cp >> 12) & 0x3F));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        }
    }

    void parse_string(std::string& out)
    {
        ++p_;  // opening quote
        for (;;) {
            if (p_ >= end_)
                error("unterminated string");
            const char c = *p_++;
            if (c == '"')
                return;
            if (static_cast<unsigned char>(c) < 0x20)
                error("control character in string");
            if (c != '\\') {
                out += c;
                continue;
            }
            if (p_ >= end_)
                error("unterminated escape");
            const char e = *p_++;
            switch (e) {
            case '"': out += '"'; break;
            case '\\': out += '\\'; break;
            case '/': out += '/'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'n': out += '\n'; break;
            case 'r': out += '\r'; break;
            case 't': out += '\t'; break;
            case 'u': {
                unsigned cp = hex4();
                if (cp >= 0xD800 && cp < 0xDC00) {
                    // a surrogate pair: the low half must follow
                    if (!(take('\\') && take('u')))
                        error("unpaired surrogate");
                    const unsigned lo = hex4();
                    if (lo < 0xDC00 || lo >= 0xE000)
                        error("unpaired surrogate");
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                } else if (cp >= 0xDC00 && cp < 0xE000) {
                    error("unpaired surrogate");
                }
                put_utf8(out, cp);
                break;
            }
            default: error("invalid escape");
            }
        }
    }
};

// ---- buffers: external files, base64 data URIs, the GLB binary chunk ----

std::vector<uint8_t> read_file(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        fail("cannot open " + path);
    f.seekg(0, std::ios::end);
    const std::streamoff size = f.tellg();
    if (size < 0)
        fail("cannot read " + path);
    f.seekg(0, std::ios::beg);
    std::vector<uint8_t> data(static_cast<size_t>(size));
    if (size > 0 && !f.read(reinterpret_cast<char*>(data.data()), size))
        fail("cannot read " + path);
    return data;
}

int base64_value(char c)
{
    if (c >= 'A' && c <= 'Z')
        return c - 'A';
    if (c >= 'a' && c <= 'z')
        return c - 'a' + 26;
    if (c >= '0' && c <= '9')
        return c - '0' + 52;
    if (c == '+')
        return 62;
    if (c == '/')
        return 63;
    return -1;
}

// RFC 4648 base64 (standard alphabet; '=' padding optional at the end).
std::vector<uint8_t> base64_decode(const char* s, size_t n)
{
    while (n > 0 && s[n - 1] == '=')
        --n;
    std::vector<uint8_t> out;
    out.reserve(n / 4 * 3 + 3);
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = 0; i < n; ++i) {
        const int v = base64_value(s[i]);
        if (v < 0)
            fail("invalid character in a base64 data URI");
        acc = (acc << 6) | uint32_t(v);
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back(uint8_t((acc >> bits) & 0xFF));
        }
    }
    return out;
}

// Relative URI references: percent escapes decoded, resolved against the glTF file's folder.
std::string resolve_uri(const std::string& base_dir, const std::string& uri)
{
    std::string path;
    for (size_t i = 0; i < uri.size(); ++i) {
        if (uri[i] == '%' && i + 2 < uri.size()) {
            auto hexv = [](char c) {
                return c >= '0' && c <= '9' ? c - '0' : c >= 'a' && c <= 'f' ? c - 'a' + 10
                                                      : c >= 'A' && c <= 'F' ? c - 'A' + 10 : -1;
            };
            const int a = hexv(uri[i + 1]), b = hexv(uri[i + 2]);
            if (a >= 0 && b >= 0) {
                path += char(a * 16 + b);
                i += 2;
                continue;
            }
        }
        path += uri[i];
    }
    if (!path.empty() && path[0] == '/')
        return path;
    return base_dir.empty() ? path : base_dir + "/" + path;
}

// ---- typed access to the glTF document ----

double num(const Json& o, const char* key, double dflt)
{
    const Json* v = o.find(key);
    if (!v)
        return dflt;
    if (v->kind != Json::Number)
        fail(std::string("glTF: '") + key + "' is not a number");
    return v->number;
}

int64_t index_of(const Json& o, const char* key, int64_t dflt, size_t limit, const char* what)
{
    const Json* v = o.find(key);
    if (!v)
        return dflt;
    if (v->kind != Json::Number || v->number != std::floor(v->number) || v->number < 0
        || v->number >= double(limit))
        fail(std::string("glTF: '") + key + "' is not a valid " + what + " index");
    return int64_t(v->number);
}

// A non-negative integer member (byte offsets, lengths, strides, counts).
size_t size_of(const Json& o, const char* key, size_t dflt)
{
    const Json* v = o.find(key);
    if (!v)
        return dflt;
    if (v->kind != Json::Number || v->number != std::floor(v->number) || v->number < 0 || v->number > 9.0e15)
        fail(std::string("glTF: '") + key + "' is not a non-negative integer");
    return size_t(v->number);
}

const std::vector<Json>& array(const Json& o, const char* key)
{
    static const std::vector<Json> empty;
    const Json* v = o.find(key);
    if (!v)
        return empty;
    if (v->kind != Json::Array)
        fail(std::string("glTF: '") + key + "' is not an array");
    return v->items;
}

// Reads up to n numbers of an array member into out (the default stays where the member is absent).
void numbers(const Json& o, const char* key, double* out, int n)
{
    const Json* v = o.find(key);
    if (!v)
        return;
    if (v->kind != Json::Array || int(v->items.size()) < n)
        fail(std::string("glTF: '") + key + "' needs " + std::to_string(n) + " numbers");
    for (int i = 0; i < n; ++i) {
        if (v->items[i].kind != Json::Number)
            fail(std::string("glTF: '") + key + "' holds a non-number");
        out[i] = v->items[i].number;
    }
}

// Column-major 4x4 affine transform in double (glTF's matrix layout).
struct Mat4
{
    double m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

    Mat4 operator*(const Mat4& b) const
    {
        Mat4 r;
        for (int c = 0; c < 4; ++c)
            for (int row = 0; row < 4; ++row) {
                double acc = 0.0;
                for (int k = 0; k < 4; ++k)
                    acc += m[k * 4 + row] * b.m[c * 4 + k];
                r.m[c * 4 + row] = acc;
            }
        return r;
    }
    void point(const float* p, float* out) const
    {
        for (int row = 0; row < 3; ++row)
            out[row] = float(m[row] * p[0] + m[4 + row] * p[1] + m[8 + row] * p[2] + m[12 + row]);
    }
    void vector(const double* v, double* out) const
    {
        for (int row = 0; row < 3; ++row)
            out[row] = m[row] * v[0] + m[4 + row] * v[1] + m[8 + row] * v[2];
    }
    // The inverse transpose of the 3x3 part (cofactors over the determinant) in the 3x3 corner.
    Mat4 inverse_transpose3() const
    {
        auto at = [&](int r, int c) { return m[c * 4 + r]; };
        const double det = det3();
        Mat4 out;
        if (det == 0.0)
            return out;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
                // cofactor C(r, c); (M^-1)^T = C / det
                out.m[c * 4 + r] = (at(r1, c1) * at(r2, c2) - at(r1, c2) * at(r2, c1)) / det;
            }
        return out;
    }
    double det3() const
    {
        return m[0] * (m[5] * m[10] - m[9] * m[6]) - m[4] * (m[1] * m[10] - m[9] * m[2])
             + m[8] * (m[1] * m[6] - m[5] * m[2]);
    }
};

// A node's local transform: 'matrix' when given, else T * R * S (glTF 2.0 section 3.5.3).
Mat4 local_transform(const Json& node)
{
    Mat4 out;
    if (node.has("matrix")) {
        numbers(node, "matrix", out.m, 16);
        return out;
    }
    double t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, sc[3] = {1, 1, 1};
    numbers(node, "translation", t, 3);
    numbers(node, "rotation", q, 4);
    numbers(node, "scale", sc, 3);
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double r[9] = {1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w),   // column 0
                         2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w),   // column 1
                         2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)};  // column 2
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 3; ++row)
            out.m[c * 4 + row] = r[c * 3 + row] * sc[c];
    out.m[12] = t[0];
    out.m[13] = t[1];
    out.m[14] = t[2];
    return out;
}

struct BufferView
{
    size_t buffer = 0, offset = 0, length = 0, stride = 0;
};

struct Accessor
{
    int64_t view = -1;      // -1: no buffer view (all zeros)
    size_t offset = 0, count = 0;
    int component = 0;      // glTF componentType
    int width = 0;          // components per element
};

size_t component_bytes(int type)
{
    switch (type) {
    case 5120: case 5121: return 1;  // BYTE, UNSIGNED_BYTE
    case 5122: case 5123: return 2;  // SHORT, UNSIGNED_SHORT
    case 5125: case 5126: return 4;  // UNSIGNED_INT, FLOAT
    default: fail("glTF: unknown accessor componentType " + std::to_string(type));
    }
}

int type_width(const std::string& t)
{
    static const std::pair<const char*, int> kinds[] = {{"SCALAR", 1}, {"VEC2", 2}, {"VEC3", 3}, {"VEC4", 4},
                                                       {"MAT2", 4}, {"MAT3", 9}, {"MAT4", 16}};
    for (const auto& k : kinds)
        if (t == k.first)
            return k.second;
    fail("glTF: unknown accessor type '" + t + "'");
}

class Document
{
public:
    Json json;
    std::vector<std::vector<uint8_t>> buffers;
    std::vector<BufferView> views;
    std::vector<Accessor> accessors;

    void load(const std::string& path)
    {
        std::vector<uint8_t> file = read_file(path);
        const size_t slash = path.find_last_of('/');
        const std::string dir = slash == std::string::npos ? std::string() : path.substr(0, slash);
        std::vector<uint8_t> glb_bin;
        bool has_glb_bin = false;
        const uint8_t* json_begin = file.data();
        size_t json_size = file.size();
        if (file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0) {
            // GLB container (glTF 2.0 section 4.4): 12-byte header, a JSON chunk, an optional BIN chunk.
            uint32_t version = 0, total = 0;
            std::memcpy(&version, file.data() + 4, 4);
            std::memcpy(&total, file.data() + 8, 4);
            if (version != 2 || total > file.size())
                fail("GLB: unsupported version or truncated file");
            size_t at = 12;
            int chunk = 0;
            while (at + 8 <= total) {
                uint32_t len = 0, type = 0;
                std::memcpy(&len, file.data() + at, 4);
                std::memcpy(&type, file.data() + at + 4, 4);
                if (size_t(len) > total - at - 8)
                    fail("GLB: chunk runs past the end of the file");
                const uint8_t* body = file.data() + at + 8;
                if (chunk == 0) {
                    if (type != 0x4E4F534Au)
                        fail("GLB: the first chunk is not JSON");
                    json_begin = body;
                    json_size = len;
                } else if (chunk == 1 && type == 0x004E4942u) {
                    glb_bin.assign(body, body + len);
                    has_glb_bin = true;
                }
                at += 8 + size_t(len);
                ++chunk;
            }
            if (chunk == 0)
                fail("GLB: no JSON chunk");
        }
        JsonReader reader(reinterpret_cast<const char*>(json_begin), reinterpret_cast<const char*>(json_begin) + json_size);
        json = reader.parse_document();
        if (json.kind != Json::Object)
            fail("glTF: the document is not a JSON object");
        const Json* asset = json.find("asset");
        const Json* version = asset ? asset->find("version") : nullptr;
        if (!version || version->kind != Json::String || version->text.compare(0, 2, "2.") != 0)
            fail("glTF: asset.version must be 2.x");
        for (const Json& e : array(json, "extensionsRequired"))
            if (e.kind == Json::String && e.text != "KHR_materials_emissive_strength" && e.text != "KHR_materials_ior"
                && e.text != "KHR_materials_transmission" && e.text != "KHR_materials_clearcoat"
                && e.text != "KHR_materials_specular" && e.text != "KHR_materials_volume"
                && e.text != "KHR_materials_sheen" && e.text != "KHR_materials_anisotropy")
                fail("glTF: required extension " + e.text + " is not supported", GBPT_ERROR_UNSUPPORTED);

        const auto& bufs = array(json, "buffers");
        for (size_t i = 0; i < bufs.size(); ++i) {
            const Json* uri = bufs[i].find("uri");
            std::vector<uint8_t> data;
            if (!uri) {
                if (i != 0 || !has_glb_bin)
                    fail("glTF: buffer " + std::to_string(i) + " has no uri");
                data = glb_bin;
            } else {
                if (uri->kind != Json::String)
                    fail("glTF: buffer uri is not a string");
                const std::string& u = uri->text;
                if (u.compare(0, 5, "data:") == 0) {
                    const size_t comma = u.find(',');
                    if (comma == std::string::npos || u.compare(comma - 7, 7, ";base64") != 0)
                        fail("glTF: only base64 data URIs are supported", GBPT_ERROR_UNSUPPORTED);
                    data = base64_decode(u.data() + comma + 1, u.size() - comma - 1);
                } else {
                    data = read_file(resolve_uri(dir, u));
                }
            }
            if (!bufs[i].has("byteLength"))
                fail("glTF: buffer " + std::to_string(i) + " without a byteLength");
            const size_t declared = size_of(bufs[i], "byteLength", 0);
            if (data.size() < declared)
                fail("glTF: buffer " + std::to_string(i) + " is shorter than its byteLength");
            data.resize(declared);
            buffers.push_back(std::move(data));
        }

        for (const Json& v : array(json, "bufferViews")) {
            BufferView bv;
            if (!v.has("buffer"))
                fail("glTF: bufferView without a buffer");
            bv.buffer = size_t(index_of(v, "buffer", 0, buffers.size(), "buffer"));
            bv.offset = size_of(v, "byteOffset", 0);
            bv.length = size_of(v, "byteLength", 0);
            bv.stride = size_of(v, "byteStride", 0);
            if (bv.offset > buffers[bv.buffer].size() || bv.length > buffers[bv.buffer].size() - bv.offset)
                fail("glTF: bufferView runs past the end of its buffer");
            views.push_back(bv);
        }

        for (const Json& a : array(json, "accessors")) {
            if (a.has("sparse"))
                fail("glTF: sparse accessors are not supported", GBPT_ERROR_UNSUPPORTED);
            Accessor acc;
            acc.view = index_of(a, "bufferView", -1, views.size(), "bufferView");
            acc.offset = size_of(a, "byteOffset", 0);
            if (!a.has("count"))
                fail("glTF: accessor without a count");
            acc.count = size_of(a, "count", 0);
            if (acc.count > (size_t(1) << 30))
                fail("glTF: accessor count too large");
            acc.component = int(num(a, "componentType", 0));
            const Json* type = a.find("type");
            if (!type || type->kind != Json::String)
                fail("glTF: accessor without a type");
            acc.width = type_width(type->text);
            const size_t elem = component_bytes(acc.component) * size_t(acc.width);
            if (acc.view >= 0 && acc.count > 0) {
                const BufferView& bv = views[size_t(acc.view)];
                const size_t stride = bv.stride ? bv.stride : elem;
                const uint64_t last = uint64_t(acc.offset) + uint64_t(stride) * (acc.count - 1) + elem;
                if (last > bv.length)
                    fail("glTF: accessor runs past the end of its bufferView");
            }
            accessors.push_back(acc);
        }
    }

    // Float VEC3 elements of an accessor (positions).
    std::vector<float> vec3f(int64_t index, const char* what) const
    {
        const Accessor& a = accessors.at(size_t(index));
        if (a.component != 5126 || a.width != 3)
            fail(std::string("glTF: ") + what + " must be a float VEC3 accessor", GBPT_ERROR_UNSUPPORTED);
        std::vector<float> out(a.count * 3, 0.0f);
        if (a.view < 0)
            return out;
        const BufferView& bv = views[size_t(a.view)];
        const uint8_t* base = buffers[bv.buffer].data() + bv.offset + a.offset;
        const size_t stride = bv.stride ? bv.stride : 12;
        for (size_t i = 0; i < a.count; ++i)
            std::memcpy(&out[i * 3], base + i * stride, 12);  // little-endian on every supported host
        return out;
    }

    // Unsigned integer SCALAR elements of an accessor (indices).
    std::vector<uint32_t> scalars_u32(int64_t index) const
    {
        const Accessor& a = accessors.at(size_t(index));
        if (a.width != 1 || (a.component != 5121 && a.component != 5123 && a.component != 5125))
            fail("glTF: indices must be an unsigned byte/short/int SCALAR accessor");
        std::vector<uint32_t> out(a.count, 0u);
        if (a.view < 0)
            return out;
        const BufferView& bv = views[size_t(a.view)];
        const size_t elem = component_bytes(a.component);
        const uint8_t* base = buffers[bv.buffer].data() + bv.offset + a.offset;
        const size_t stride = bv.stride ? bv.stride : elem;
        for (size_t i = 0; i < a.count; ++i) {
            const uint8_t* e = base + i * stride;
            if (elem == 1) {
                out[i] = e[0];
            } else if (elem == 2) {
                uint16_t v;
                std::memcpy(&v, e, 2);
                out[i] = v;
            } else {
                std::memcpy(&out[i], e, 4);
            }
        }
        return out;
    }
};

// ---- materials ----

// CPUMaterial's defaults (src/HostDeviceCommon/Material/MaterialCPU.h:209-300) in the fields of
// gbpt_principled_material.
gbpt_principled_material cpu_material_defaults()
{
    gbpt_principled_material m;
    std::memset(&m, 0, sizeof m);
    auto rgb = [](float* c, float v) { c[0] = c[1] = c[2] = v; };
    rgb(m.base_color, 1.0f);
    m.roughness = 0.3f;
    rgb(m.metallic_F82, 1.0f);
    m.metallic_F90_falloff_exponent = 5.0f;
    rgb(m.metallic_F90, 1.0f);
    m.second_roughness = 0.5f;
    m.specular = 1.0f;
    rgb(m.specular_color, 1.0f);
    m.specular_tint = 1.0f;
    m.coat_roughening = 1.0f;
    rgb(m.coat_medium_absorption, 1.0f);
    m.coat_medium_thickness = 5.0f;
    m.coat_darkening = 1.0f;
    m.coat_ior = 1.5f;
    m.ior = 1.4f;
    rgb(m.absorption_color, 1.0f);
    m.absorption_at_distance = 1.0f;
    m.diffuse_lobe = GBPT_DIFFUSE_LAMBERTIAN;
    m.oren_nayar_sigma = 0.34906585039886591538f;  // 20 degrees
    m.thin_film_ior = 1.3f;
    m.thin_film_thickness = 500.0f;
    m.thin_film_base_ior_override = 1.0f;
    m.dispersion_abbe_number = 20.0f;
    return m;
}

float clamp01(float v) { return std::fmin(1.0f, std::fmax(0.0f, v)); }
float clampf(float lo, float hi, float v) { return std::fmin(hi, std::fmax(lo, v)); }

// The clamps of CPUMaterial::make_safe (src/HostDeviceCommon/Material/MaterialCPU.h:156-207) on the
// fields this record holds.
void make_safe(gbpt_principled_material& m)
{
    for (int k = 0; k < 3; ++k) {
        m.base_color[k] = clamp01(m.base_color[k]);
        m.metallic_F82[k] = clamp01(m.metallic_F82[k]);
        m.metallic_F90[k] = clamp01(m.metallic_F90[k]);
        m.specular_color[k] = clamp01(m.specular_color[k]);
        m.coat_medium_absorption[k] = clamp01(m.coat_medium_absorption[k]);
        m.absorption_color[k] = clamp01(std::fmax(m.absorption_color[k], 1.0f / 512.0f));
        m.emission[k] = std::fmax(0.0f, m.emission[k]);
    }
    m.metallic = clamp01(m.metallic);
    m.anisotropy = clamp01(m.anisotropy);
    m.anisotropy_rotation = clamp01(m.anisotropy_rotation);
    m.second_roughness_weight = clamp01(m.second_roughness_weight);
    m.second_roughness = clamp01(m.second_roughness);
    m.specular = clamp01(m.specular);
    m.specular_tint = clamp01(m.specular_tint);
    m.specular_darkening = clamp01(m.specular_darkening);
    m.coat = clamp01(m.coat);
    m.coat_roughness = clampf(1.0e-4f, 1.0f, m.coat_roughness);  // MaterialConstants::ROUGHNESS_CLAMP
    m.coat_roughening = clamp01(m.coat_roughening);
    m.coat_darkening = clamp01(m.coat_darkening);
    m.coat_anisotropy = clamp01(m.coat_anisotropy);
    m.coat_anisotropy_rotation = clamp01(m.coat_anisotropy_rotation);
    m.sheen = clamp01(m.sheen);
    m.specular_transmission = clamp01(m.specular_transmission);
    m.absorption_at_distance = std::fmax(m.absorption_at_distance, 1.0e-4f);
}

const Json* extension(const Json& mat, const char* name)
{
    const Json* ext = mat.find("extensions");
    return ext ? ext->find(name) : nullptr;
}

// One glTF material through read_material_properties (src/Scene/SceneParser.cpp:391-438): the keys
// ASSIMP's glTF 2 importer always fills (diffuse colour <- baseColorFactor, emissive colour <-
// emissiveFactor, metallic and roughness factors with the glTF defaults of 1) are always read;
// the extension keys are read only when their extension is on the material, as the reference's
// Get() calls leave a field at CPUMaterial's default when the key is missing. Emission is
// clamped by make_safe first and then scaled by the emissive strength, as the reference bakes
// emission_strength into the emission it uploads.
gbpt_principled_material material_from_gltf(const Json& mat)
{
    gbpt_principled_material m = cpu_material_defaults();
    double base[4] = {1, 1, 1, 1};
    double metallic = 1.0, roughness = 1.0;
    if (const Json* pbr = mat.find("pbrMetallicRoughness")) {
        numbers(*pbr, "baseColorFactor", base, 4);
        metallic = num(*pbr, "metallicFactor", 1.0);
        roughness = num(*pbr, "roughnessFactor", 1.0);
    }
    for (int k = 0; k < 3; ++k)
        m.base_color[k] = float(base[k]);
    m.metallic = float(metallic);
    m.roughness = float(roughness);
    double emissive[3] = {0, 0, 0};
    numbers(mat, "emissiveFactor", emissive, 3);
    for (int k = 0; k < 3; ++k)
        m.emission[k] = float(emissive[k]);
    float strength = 1.0f;
    if (const Json* e = extension(mat, "KHR_materials_emissive_strength"))
        strength = float(num(*e, "emissiveStrength", 1.0));
    if (const Json* e = extension(mat, "KHR_materials_anisotropy"))
        m.anisotropy = float(num(*e, "anisotropyStrength", 0.0));
    if (extension(mat, "KHR_materials_sheen"))
        m.sheen = 1.0f;  // the reference turns sheen fully on when the sheen colour key exists
    if (const Json* e = extension(mat, "KHR_materials_specular")) {
        m.specular = float(num(*e, "specularFactor", 1.0));
        m.specular_tint = 1.0f;
        m.specular_color[0] = m.specular_color[1] = m.specular_color[2] = 1.0f;
    }
    if (const Json* e = extension(mat, "KHR_materials_clearcoat")) {
        m.coat = float(num(*e, "clearcoatFactor", 0.0));
        m.coat_roughness = float(num(*e, "clearcoatRoughnessFactor", 0.0));
    }
    if (const Json* e = extension(mat, "KHR_materials_ior"))
        m.ior = float(num(*e, "ior", 1.5));
    if (const Json* e = extension(mat, "KHR_materials_transmission"))
        m.specular_transmission = float(num(*e, "transmissionFactor", 0.0));
    if (const Json* e = extension(mat, "KHR_materials_volume")) {
        double color[3] = {1, 1, 1};
        numbers(*e, "attenuationColor", color, 3);
        for (int k = 0; k < 3; ++k)
            m.absorption_color[k] = float(color[k]);
        // the extension's default distance is +infinity (no absorption); the largest float keeps
        // the record finite
        m.absorption_at_distance = e->has("attenuationDistance") ? float(num(*e, "attenuationDistance", 0.0)) : 3.4028235e38f;
    }
    make_safe(m);
    for (int k = 0; k < 3; ++k)
        m.emission[k] *= strength;
    return m;
}

}  // namespace

// ---- the loaded scene ----

struct gbpt_gltf
{
    std::vector<float> positions;          // world space, 3 per vertex
    std::vector<float> normals;            // world space, 3 per vertex (zero: none); empty when no primitive has any
    std::vector<int32_t> indices;          // 3 per triangle
    std::vector<int32_t> material_indices; // 1 per triangle
    std::vector<gbpt_principled_material> materials;
    gbpt_gltf_camera camera{};
};

namespace {

void normalise(double* v)
{
    const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (n > 0.0)
        for (int k = 0; k < 3; ++k)
            v[k] /= n;
}

class SceneBuilder
{
public:
    SceneBuilder(const Document& doc, gbpt_gltf& out) : doc_(doc), out_(out) {}

    void build()
    {
        const Json& j = doc_.json;
        const auto& nodes = array(j, "nodes");
        for (const Json& m : array(j, "materials"))
            out_.materials.push_back(material_from_gltf(m));

        // the default scene's root nodes ('scene', else scene 0); a file without scenes shows every
        // node that no other node lists as a child
        std::vector<size_t> roots;
        const auto& scenes = array(j, "scenes");
        if (!scenes.empty()) {
            const Json& sc = scenes[size_t(index_of(j, "scene", 0, scenes.size(), "scene"))];
            for (const Json& n : array(sc, "nodes"))
                roots.push_back(node_index(n, nodes.size()));
        } else {
            std::vector<char> child(nodes.size(), 0);
            for (const Json& n : nodes)
                for (const Json& c : array(n, "children"))
                    child[node_index(c, nodes.size())] = 1;
            for (size_t i = 0; i < nodes.size(); ++i)
                if (!child[i])
                    roots.push_back(i);
        }

        // depth-first, children in file order; the depth bound catches cycles
        struct Item { size_t node; Mat4 parent; size_t depth; };
        std::vector<Item> stack;
        for (size_t r = roots.size(); r-- > 0;)
            stack.push_back({roots[r], Mat4(), 0});
        while (!stack.empty()) {
            const Item it = stack.back();
            stack.pop_back();
            if (it.depth > nodes.size())
                fail("glTF: the node hierarchy has a cycle");
            const Json& node = nodes[it.node];
            const Mat4 world = it.parent * local_transform(node);
            if (node.has("mesh"))
                add_mesh(size_t(index_of(node, "mesh", 0, array(j, "meshes").size(), "mesh")), world);
            if (node.has("camera"))
                consider_camera(size_t(index_of(node, "camera", 0, array(j, "cameras").size(), "camera")), world);
            const auto& children = array(node, "children");
            for (size_t c = children.size(); c-- > 0;)
                stack.push_back({node_index(children[c], nodes.size()), world, it.depth + 1});
        }
    }

private:
    const Document& doc_;
    gbpt_gltf& out_;
    int32_t default_material_ = -1;
    int64_t camera_index_ = -1;
    bool any_normals_ = false;

    static size_t node_index(const Json& v, size_t n)
    {
        if (v.kind != Json::Number || v.number != std::floor(v.number) || v.number < 0 || v.number >= double(n))
            fail("glTF: invalid node index");
        return size_t(v.number);
    }

    int32_t default_material()
    {
        // a primitive without a material: the glTF default material (an empty material object)
        if (default_material_ < 0) {
            default_material_ = int32_t(out_.materials.size());
            out_.materials.push_back(material_from_gltf(Json()));
        }
        return default_material_;
    }

    void add_mesh(size_t mesh_index, const Mat4& world)
    {
        const Json& mesh = array(doc_.json, "meshes")[mesh_index];
        const bool mirrored = world.det3() < 0.0;
        for (const Json& prim : array(mesh, "primitives")) {
            const size_t mode = size_of(prim, "mode", 4);
            if (mode < 4)
                continue;  // points and lines carry no surface
            if (mode > 6)
                fail("glTF: unknown primitive mode " + std::to_string(mode));
            const Json* attrs = prim.find("attributes");
            if (!attrs || !attrs->has("POSITION"))
                fail("glTF: primitive without POSITION");
            const std::vector<float> pos = doc_.vec3f(index_of(*attrs, "POSITION", 0, doc_.accessors.size(), "accessor"), "POSITION");
            const size_t nv = pos.size() / 3;
            std::vector<float> nrm;
            if (attrs->has("NORMAL")) {
                nrm = doc_.vec3f(index_of(*attrs, "NORMAL", 0, doc_.accessors.size(), "accessor"), "NORMAL");
                if (nrm.size() != pos.size())
                    fail("glTF: NORMAL and POSITION counts differ");
            }
            std::vector<uint32_t> idx;
            if (prim.has("indices")) {
                idx = doc_.scalars_u32(index_of(prim, "indices", 0, doc_.accessors.size(), "accessor"));
                for (uint32_t i : idx)
                    if (i >= nv)
                        fail("glTF: vertex index out of range");
            } else {
                idx.resize(nv);
                for (size_t i = 0; i < nv; ++i)
                    idx[i] = uint32_t(i);
            }
            const int32_t material = prim.has("material")
                ? int32_t(index_of(prim, "material", 0, array(doc_.json, "materials").size(), "material"))
                : default_material();

            const size_t base = out_.positions.size() / 3;
            if (base + nv > size_t(INT32_MAX))
                fail("glTF: more than 2^31 vertices", GBPT_ERROR_UNSUPPORTED);
            out_.positions.resize((base + nv) * 3);
            for (size_t v = 0; v < nv; ++v)
                world.point(&pos[v * 3], &out_.positions[(base + v) * 3]);
            // normals to world space by the inverse transpose of the node's 3x3 part, normalised
            // (what ASSIMP's pre-transform step does to them); zero where the primitive has none
            if (!nrm.empty() && !any_normals_) {
                out_.normals.assign(base * 3, 0.0f);  // earlier primitives had none
                any_normals_ = true;
            }
            if (any_normals_) {
                out_.normals.resize((base + nv) * 3, 0.0f);
                if (!nrm.empty()) {
                    const Mat4 it = world.inverse_transpose3();
                    for (size_t v = 0; v < nv; ++v) {
                        const double n[3] = {nrm[v * 3], nrm[v * 3 + 1], nrm[v * 3 + 2]};
                        double w[3];
                        it.vector(n, w);
                        normalise(w);
                        for (int k = 0; k < 3; ++k)
                            out_.normals[(base + v) * 3 + k] = float(w[k]);
                    }
                }
            }

            // triangles of the primitive (glTF 2.0 section 3.7.2.1: lists, strips, fans)
            auto emit = [&](uint32_t a, uint32_t b, uint32_t c) {
                if (mirrored)
                    std::swap(b, c);
                out_.indices.push_back(int32_t(base + a));
                out_.indices.push_back(int32_t(base + b));
                out_.indices.push_back(int32_t(base + c));
                out_.material_indices.push_back(material);
            };
            const size_t n = idx.size();
            if (mode == 4) {
                for (size_t t = 0; t + 2 < n; t += 3)
                    emit(idx[t], idx[t + 1], idx[t + 2]);
            } else if (mode == 5) {
                for (size_t t = 0; t + 2 < n; ++t)
                    if (t % 2 == 0)
                        emit(idx[t], idx[t + 1], idx[t + 2]);
                    else
                        emit(idx[t + 1], idx[t], idx[t + 2]);
            } else {
                for (size_t t = 1; t + 1 < n; ++t)
                    emit(idx[t], idx[t + 1], idx[0]);
            }
            if (out_.indices.size() / 3 > size_t(INT32_MAX))
                fail("glTF: more than 2^31 triangles", GBPT_ERROR_UNSUPPORTED);
        }
    }

    // The camera: the perspective camera with the lowest index in 'cameras' (the reference takes
    // aiScene::mCameras[0], src/Scene/SceneParser.cpp:227-262) seen from the first node that
    // carries it. Position is the node's origin, forward its -Z axis and up its +Y axis in world
    // space (the glTF camera convention).
    void consider_camera(size_t index, const Mat4& world)
    {
        if (camera_index_ >= 0 && int64_t(index) >= camera_index_)
            return;
        const Json& cam = array(doc_.json, "cameras")[index];
        const Json* type = cam.find("type");
        const Json* persp = cam.find("perspective");
        if (!type || type->kind != Json::String || type->text != "perspective" || !persp)
            return;
        camera_index_ = int64_t(index);
        gbpt_gltf_camera& c = out_.camera;
        c.present = 1;
        const float origin[3] = {0, 0, 0};
        world.point(origin, c.position);
        const double fwd_local[3] = {0, 0, -1}, up_local[3] = {0, 1, 0};
        double fwd[3], up[3];
        world.vector(fwd_local, fwd);
        world.vector(up_local, up);
        normalise(fwd);
        normalise(up);
        for (int k = 0; k < 3; ++k) {
            c.forward[k] = float(fwd[k]);
            c.up[k] = float(up[k]);
        }
        c.yfov = float(num(*persp, "yfov", 0.0));
        c.aspect_ratio = float(num(*persp, "aspectRatio", 0.0));
        c.znear = float(num(*persp, "znear", 0.0));
        c.zfar = float(num(*persp, "zfar", 0.0));
    }
};

}  // namespace

extern "C" {

gbpt_status gbpt_gltf_load(const char* path, gbpt_gltf** out)
{
    if (!out)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!path)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "path is NULL");
    try {
        std::unique_ptr<gbpt_gltf> g(new gbpt_gltf());
        Document doc;
        doc.load(path);
        SceneBuilder(doc, *g).build();
        *out = g.release();
        return GBPT_OK;
    } catch (const GltfError& e) {
        return gbpt::set_error(e.status, std::string(path) + ": " + e.msg);
    } catch (const std::bad_alloc&) {
        return gbpt::set_error(GBPT_ERROR_OOM, "host allocation failed while loading " + std::string(path));
    } catch (const std::exception& e) {
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, std::string(path) + ": " + e.what());
    }
}

gbpt_status gbpt_gltf_scene_desc(const gbpt_gltf* g, gbpt_scene_desc* out)
{
    if (!g || !out)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "gltf or out is NULL");
    std::memset(out, 0, sizeof *out);
    out->positions = g->positions.data();
    out->n_vertices = int64_t(g->positions.size() / 3);
    out->indices = g->indices.data();
    out->n_triangles = int64_t(g->indices.size() / 3);
    out->material_indices = g->material_indices.data();
    out->materials = nullptr;
    out->n_materials = int32_t(g->materials.size());
    out->principled_materials = g->materials.data();
    out->vertex_normals = g->normals.empty() ? nullptr : g->normals.data();
    return GBPT_OK;
}

gbpt_status gbpt_gltf_get_camera(const gbpt_gltf* g, gbpt_gltf_camera* out)
{
    if (!g || !out)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "gltf or out is NULL");
    *out = g->camera;
    return GBPT_OK;
}

gbpt_status gbpt_gltf_destroy(gbpt_gltf* g)
{
    delete g;
    return GBPT_OK;
}

}  // extern "C"
