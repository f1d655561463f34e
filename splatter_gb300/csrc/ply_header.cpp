// Validated splat-file header (host only).
//
// The reference's Scene::parse_file_header (scene.rs:197-213) reads lines until "end_header\n",
// takes the `element vertex` count, and keeps the header length in a u16; Scene::load_chunk
// (scene.rs:216-224) then reads 248-byte records of 62 little-endian floats (SerializedSplat,
// scene.rs:15-24) right after the header.  Any other layout is silently misread (or panics on a CRLF
// header).  spl_validate_file_header checks that the file really has that layout before a load:
// binary little-endian PLY, the vertex element first, exactly 62 float properties (in the standard
// 3D-Gaussian order when names are checked), LF or CRLF lines, and a body long enough for the
// declared count.  Every failure is SPL_ERR_IO with a message naming the offending line.
#include <cstdio>
#include <cstring>
#include <string>

#include "spl_internal.h"

namespace {

// SerializedSplat's fields in file order: center[3], n[3], color[48] (f_dc_0..2 then f_rest_0..44),
// alpha, scale[3], rotation[4].
std::string standard_property_name(int k) {
    static const char* head[6] = {"x", "y", "z", "nx", "ny", "nz"};
    if (k < 6) return head[k];
    if (k < 9) return "f_dc_" + std::to_string(k - 6);
    if (k < 54) return "f_rest_" + std::to_string(k - 9);
    if (k == 54) return "opacity";
    if (k < 58) return "scale_" + std::to_string(k - 55);
    return "rot_" + std::to_string(k - 58);
}

// Splits off the next whitespace-separated word of `p`; returns false at the end of the line.
bool next_word(const char*& p, std::string& w) {
    while (*p == ' ' || *p == '\t') ++p;
    if (!*p) return false;
    const char* b = p;
    while (*p && *p != ' ' && *p != '\t') ++p;
    w.assign(b, p);
    return true;
}

}  // namespace

extern "C" int spl_validate_file_header(const char* path, int check_names, uint32_t* header_bytes,
                                        uint64_t* splat_count) {
    using spl::fail;
    if (!path || !header_bytes || !splat_count) return fail(SPL_ERR_INVALID, "NULL argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(SPL_ERR_IO, "cannot open %s", path);
    struct Closer {
        FILE* f;
        ~Closer() { std::fclose(f); }
    } closer{f};
    char buf[4096];
    uint64_t pos = 0;
    int lineno = 0;
    bool have_format = false, in_vertex = false, vertex_done = false, ended = false;
    uint64_t count = 0;
    int props = 0;
    while (std::fgets(buf, sizeof(buf), f)) {
        ++lineno;
        size_t len = std::strlen(buf);
        pos += len;
        if (len == 0 || buf[len - 1] != '\n') return fail(SPL_ERR_IO, "%s: header line %d is not terminated", path, lineno);
        buf[--len] = '\0';
        if (len && buf[len - 1] == '\r') buf[--len] = '\0';  // CRLF
        const std::string line(buf);
        if (lineno == 1) {
            if (line != "ply") return fail(SPL_ERR_IO, "%s: not a PLY file (first line '%s')", path, buf);
            continue;
        }
        const char* p = buf;
        std::string kw;
        if (!next_word(p, kw)) continue;  // blank line
        if (kw == "comment" || kw == "obj_info") continue;
        if (kw == "end_header") {
            ended = true;
            break;
        }
        if (kw == "format") {
            std::string fmt, ver;
            if (!next_word(p, fmt) || !next_word(p, ver) || fmt != "binary_little_endian" || ver != "1.0")
                return fail(SPL_ERR_IO, "%s: line %d: only 'format binary_little_endian 1.0' is supported ('%s')", path,
                            lineno, buf);
            have_format = true;
            continue;
        }
        if (kw == "element") {
            std::string name, num;
            if (!next_word(p, name) || !next_word(p, num))
                return fail(SPL_ERR_IO, "%s: line %d: malformed element line '%s'", path, lineno, buf);
            if (in_vertex) {
                in_vertex = false;
                vertex_done = true;
            }
            if (name == "vertex") {
                if (vertex_done) return fail(SPL_ERR_IO, "%s: line %d: a second vertex element", path, lineno);
                char* endp = nullptr;
                count = std::strtoull(num.c_str(), &endp, 10);
                if (num.empty() || *endp != '\0' || num[0] == '-')
                    return fail(SPL_ERR_IO, "%s: line %d: bad vertex count '%s'", path, lineno, num.c_str());
                in_vertex = true;
            } else if (!vertex_done) {
                // its data would precede the vertex records, which the loader reads right after the header
                return fail(SPL_ERR_IO, "%s: line %d: element '%s' before the vertex element", path, lineno,
                            name.c_str());
            }
            continue;
        }
        if (kw == "property") {
            if (!in_vertex) {
                if (vertex_done) continue;  // a property of an element after the vertex data
                return fail(SPL_ERR_IO, "%s: line %d: property outside an element", path, lineno);
            }
            std::string type, name;
            if (!next_word(p, type) || !next_word(p, name))
                return fail(SPL_ERR_IO, "%s: line %d: malformed property line '%s'", path, lineno, buf);
            if (type != "float" && type != "float32")
                return fail(SPL_ERR_IO, "%s: line %d: vertex property '%s' is '%s', the loader reads 32-bit floats", path,
                            lineno, name.c_str(), type.c_str());
            if (props >= 62) return fail(SPL_ERR_IO, "%s: line %d: more than 62 vertex properties", path, lineno);
            if (check_names && name != standard_property_name(props))
                return fail(SPL_ERR_IO, "%s: line %d: vertex property %d is '%s', expected '%s'", path, lineno, props,
                            name.c_str(), standard_property_name(props).c_str());
            ++props;
            continue;
        }
        return fail(SPL_ERR_IO, "%s: line %d: unknown header line '%s'", path, lineno, buf);
    }
    if (!ended) return fail(SPL_ERR_IO, "%s: no end_header line", path);
    if (!have_format) return fail(SPL_ERR_IO, "%s: no format line", path);
    if (!in_vertex && !vertex_done) return fail(SPL_ERR_IO, "%s: no vertex element", path);
    if (props != 62) return fail(SPL_ERR_IO, "%s: %d vertex properties, the loader reads 62", path, props);
    if (pos > 0xFFFFFFFFull) return fail(SPL_ERR_IO, "%s: header longer than 4 GiB", path);
    if (std::fseek(f, 0, SEEK_END) != 0) return fail(SPL_ERR_IO, "%s: seek failed", path);
    const long end = std::ftell(f);
    if (end < 0) return fail(SPL_ERR_IO, "%s: cannot size the file", path);
    const uint64_t body = (uint64_t)end - pos;
    if (count > body / 248u)
        return fail(SPL_ERR_IO, "%s: the header declares %llu splats, the file holds %llu", path,
                    (unsigned long long)count, (unsigned long long)(body / 248u));
    *header_bytes = (uint32_t)pos;
    *splat_count = count;
    return SPL_OK;
}
