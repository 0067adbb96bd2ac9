// .mscene scene files (host code): a reader of the Cap'n Proto packed
// encoding written for the reference's schema src/micropolis/mscene.capnp,
// and Scene::draw (src/micropolis/Scene.cpp:89-197) over the C ABI.
//
// Encoding (the published Cap'n Proto format, nothing else is needed):
//  * packed stream: every 8-byte word is a tag byte whose bit i says that
//    byte i is nonzero and follows; tag 0x00 is followed by a count of extra
//    zero words, tag 0xFF by the 8 bytes and a count of raw words copied as is;
//  * message: uint32 (segments - 1), uint32 size of each segment in words,
//    padding to a word, then the segments;
//  * pointers (64-bit, little endian): bits 0-1 kind (0 struct, 1 list,
//    2 far), bits 2-31 signed word offset from the end of the pointer;
//    struct: bits 32-47 data words, 48-63 pointer words; list: bits 32-34
//    element size (2 byte, 4 four bytes, 7 composite), bits 35-63 count
//    (composite: words, the element count is in the tag word that precedes
//    the elements); far: bit 2 double-far, bits 3-31 landing-pad offset,
//    bits 32-63 segment.
//
// Field layout of mscene.capnp as the schema compiler assigns it (fields in
// ordinal order, each in the first free slot of its size):
//   Scene       ptr0 meshes, ptr1 lights, ptr2 objects, ptr3 cameras
//   Camera      ptr0 name, ptr1 transform; f32 #0 near, #1 far, #2 fovy
//   LightSource ptr0 name, ptr1 transform, ptr2 color; f32 #0 intensity, u16 #2 type
//   Object      ptr0 name, ptr1 transform, ptr2 meshname, ptr3 color
//   Mesh        ptr0 name, ptr1 positions (List(Float32)); u16 #0 type
//   Transform   ptr0 translation, ptr1 rotation
//   Vec3        f32 #0 x, #1 y, #2 z;  Quaternion f32 #0 r, #1 i, #2 j, #3 k
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mp_core.h"

struct mp_scene {
    struct Mesh {
        std::string name;
        int32_t type = 0;
        std::vector<float> xyz;
    };
    struct Object {
        std::string name;
        float translation[3] = {0, 0, 0};
        float rotation[4] = {1, 0, 0, 0};   // r, i, j, k
        std::string meshname;
        int32_t mesh = -1;
        float color[3] = {0, 0, 0};
    };
    struct Camera {
        std::string name;
        float translation[3] = {0, 0, 0};
        float rotation[4] = {1, 0, 0, 0};
        float near_plane = 0, far_plane = 0, fovy = 0;
    };
    std::vector<Mesh> meshes;
    std::vector<Object> objects;
    std::vector<Camera> cameras;
    int32_t lights = 0;
    std::string err;
    uint64_t uid = 0;   // distinct for every scene read in this process
};

namespace {

// ---------------------------------------------------------------------------
// packed stream -> words

bool unpack(const uint8_t* p, size_t n, std::vector<uint64_t>& out) {
    size_t i = 0;
    while (i < n) {
        const uint8_t tag = p[i++];
        uint8_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int b = 0; b < 8; ++b)
            if (tag & (1u << b)) {
                if (i >= n) return false;
                w[b] = p[i++];
            }
        uint64_t v;
        std::memcpy(&v, w, 8);
        out.push_back(v);
        if (tag == 0x00) {
            if (i >= n) return false;
            out.insert(out.end(), p[i++], 0ull);
        } else if (tag == 0xFF) {
            if (i >= n) return false;
            const size_t words = p[i++];
            if (i + 8 * words > n) return false;
            for (size_t k = 0; k < words; ++k) {
                std::memcpy(&v, p + i, 8);
                out.push_back(v);
                i += 8;
            }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// message and pointers

struct Message {
    std::vector<std::pair<size_t, size_t>> seg;   // (first word, words) in `w`
    std::vector<uint64_t> w;
    size_t budget = 1ull << 28;                     // words that may still be read (traversal limit)
};

struct Ref {      // a resolved pointer: the pointer word and the target's position
    int seg = -1;
    size_t at = 0;
    uint64_t v = 0;
};

bool parse_frame(Message& m) {
    if (m.w.empty()) return false;
    const uint32_t nseg = (uint32_t)(m.w[0] & 0xffffffffu) + 1;
    if (nseg == 0 || nseg > 1024) return false;
    const size_t table_words = (4 + 4 * (size_t)nseg + 7) / 8;
    if (m.w.size() < table_words) return false;
    const uint8_t* tb = reinterpret_cast<const uint8_t*>(m.w.data());
    size_t pos = table_words;
    for (uint32_t s = 0; s < nseg; ++s) {
        uint32_t size;
        std::memcpy(&size, tb + 4 + 4 * s, 4);
        if (pos + size > m.w.size()) return false;
        m.seg.emplace_back(pos, size);
        pos += size;
    }
    return true;
}

bool word(const Message& m, int seg, size_t at, uint64_t& v) {
    if (seg < 0 || (size_t)seg >= m.seg.size() || at >= m.seg[(size_t)seg].second) return false;
    v = m.w[m.seg[(size_t)seg].first + at];
    return true;
}

int64_t ptr_offset(uint64_t v) { return (int64_t)(int32_t)(uint32_t)(v & 0xffffffffu) >> 2; }

// A target position inside segment seg (the end of the segment included).
bool target(const Message& m, int seg, int64_t at, Ref& r) {
    if (seg < 0 || (size_t)seg >= m.seg.size() || at < 0 || (uint64_t)at > m.seg[(size_t)seg].second) return false;
    r.seg = seg;
    r.at = (size_t)at;
    return true;
}

// Follows the pointer stored at (seg, at); r.seg = -1 for a null pointer.
bool follow(const Message& m, int seg, size_t at, Ref& r) {
    uint64_t v;
    if (!word(m, seg, at, v)) return false;
    r = Ref{};
    if (v == 0) return true;
    if ((v & 3) == 2) {
        const bool dbl = (v >> 2) & 1;
        const size_t pad = (size_t)((v >> 3) & 0x1fffffffu);
        const int pseg = (int)(v >> 32);
        uint64_t p0;
        if (!word(m, pseg, pad, p0)) return false;
        if (!dbl) {
            if ((p0 & 3) == 2 || (p0 & 3) == 3) return false;
            r.v = p0;
            return target(m, pseg, (int64_t)pad + 1 + ptr_offset(p0), r);
        }
        uint64_t tag;
        if (!word(m, pseg, pad + 1, tag) || (p0 & 7) != 2 || (tag & 3) >= 2) return false;
        r.v = tag;
        return target(m, (int)(p0 >> 32), (int64_t)((p0 >> 3) & 0x1fffffffu), r);
    }
    if ((v & 3) == 3) return false;   // capabilities do not occur in a scene file
    r.v = v;
    return target(m, seg, (int64_t)at + 1 + ptr_offset(v), r);
}

struct Struct {
    const Message* m = nullptr;
    int seg = -1;
    size_t data = 0, ptrs = 0;
    uint32_t dwords = 0, pwords = 0;
    bool null() const { return seg < 0; }
    uint32_t u32(int i) const {   // 32-bit field #i, 0 beyond the data section
        if (null() || (size_t)(i + 1) * 4 > (size_t)dwords * 8) return 0;
        const uint8_t* b = reinterpret_cast<const uint8_t*>(&m->w[m->seg[(size_t)seg].first + data]);
        uint32_t v;
        std::memcpy(&v, b + 4 * i, 4);
        return v;
    }
    float f32(int i) const {
        uint32_t u = u32(i);
        float f;
        std::memcpy(&f, &u, 4);
        return f;
    }
    uint16_t u16(int i) const {
        if (null() || (size_t)(i + 1) * 2 > (size_t)dwords * 8) return 0;
        const uint8_t* b = reinterpret_cast<const uint8_t*>(&m->w[m->seg[(size_t)seg].first + data]);
        uint16_t v;
        std::memcpy(&v, b + 2 * i, 2);
        return v;
    }
};

bool charge(Message& m, size_t words) {
    if (words > m.budget) return false;
    m.budget -= words;
    return true;
}

bool make_struct(Message& m, const Ref& r, Struct& s) {
    s = Struct{};
    s.m = &m;
    if (r.seg < 0) return true;
    if ((r.v & 3) != 0) return false;
    s.seg = r.seg;
    s.dwords = (uint32_t)((r.v >> 32) & 0xffff);
    s.pwords = (uint32_t)(r.v >> 48);
    s.data = r.at;
    s.ptrs = r.at + s.dwords;
    if (s.ptrs + s.pwords > m.seg[(size_t)r.seg].second) return false;
    return charge(m, s.dwords + s.pwords);
}

bool get_struct(Message& m, const Struct& parent, int i, Struct& out) {
    out = Struct{};
    out.m = &m;
    if (parent.null() || (uint32_t)i >= parent.pwords) return true;
    Ref r;
    if (!follow(m, parent.seg, parent.ptrs + (size_t)i, r)) return false;
    return make_struct(m, r, out);
}

// List(struct): the elements, in order.
bool get_struct_list(Message& m, const Struct& parent, int i, std::vector<Struct>& out) {
    out.clear();
    if (parent.null() || (uint32_t)i >= parent.pwords) return true;
    Ref r;
    if (!follow(m, parent.seg, parent.ptrs + (size_t)i, r)) return false;
    if (r.seg < 0) return true;
    if ((r.v & 3) != 1 || ((r.v >> 32) & 7) != 7) return false;
    const size_t words = (size_t)(r.v >> 35);
    uint64_t tag;
    if (!word(m, r.seg, r.at, tag) || (tag & 3) != 0) return false;
    const size_t n = (size_t)((tag >> 2) & 0x3fffffffu);
    const uint32_t dw = (uint32_t)((tag >> 32) & 0xffff), pw = (uint32_t)(tag >> 48);
    if ((size_t)(dw + pw) * n > words || r.at + 1 + words > m.seg[(size_t)r.seg].second) return false;
    if (!charge(m, words + 1)) return false;
    for (size_t k = 0; k < n; ++k) {
        Struct s;
        s.m = &m;
        s.seg = r.seg;
        s.dwords = dw;
        s.pwords = pw;
        s.data = r.at + 1 + k * (dw + pw);
        s.ptrs = s.data + dw;
        out.push_back(s);
    }
    return true;
}

// List of `bytes`-wide primitives: pointer to the first element and the count.
bool get_prim_list(Message& m, const Struct& parent, int i, int size_code, const uint8_t*& p, size_t& n) {
    p = nullptr;
    n = 0;
    if (parent.null() || (uint32_t)i >= parent.pwords) return true;
    Ref r;
    if (!follow(m, parent.seg, parent.ptrs + (size_t)i, r)) return false;
    if (r.seg < 0) return true;
    if ((r.v & 3) != 1 || (int)((r.v >> 32) & 7) != size_code) return false;
    n = (size_t)(r.v >> 35);
    const size_t bytes = size_code == 2 ? n : size_code == 3 ? 2 * n : size_code == 4 ? 4 * n : 8 * n;
    const size_t words = (bytes + 7) / 8;
    if (r.at + words > m.seg[(size_t)r.seg].second || !charge(m, words)) return false;
    p = reinterpret_cast<const uint8_t*>(&m.w[m.seg[(size_t)r.seg].first + r.at]);
    return true;
}

bool get_text(Message& m, const Struct& parent, int i, std::string& out) {
    const uint8_t* p;
    size_t n;
    out.clear();
    if (!get_prim_list(m, parent, i, 2, p, n)) return false;
    if (n == 0) return true;
    if (p[n - 1] != 0) return false;   // Text ends with a NUL byte
    out.assign(reinterpret_cast<const char*>(p), n - 1);
    return true;
}

bool get_transform(Message& m, const Struct& parent, int i, float t[3], float q[4]) {
    Struct tr, tv, rq;
    if (!get_struct(m, parent, i, tr) || !get_struct(m, tr, 0, tv) || !get_struct(m, tr, 1, rq)) return false;
    for (int k = 0; k < 3; ++k) t[k] = tv.f32(k);
    for (int k = 0; k < 4; ++k) q[k] = rq.f32(k);
    return true;
}

bool decode(Message& m, mp_scene& s) {
    Ref root;
    if (!follow(m, 0, 0, root)) return false;
    Struct sc;
    if (!make_struct(m, root, sc) || sc.null()) return false;
    std::vector<Struct> list;
    // meshes (Scene.cpp:135-159): positions flattened, three floats per point
    if (!get_struct_list(m, sc, 0, list)) return false;
    for (const Struct& e : list) {
        mp_scene::Mesh mesh;
        if (!get_text(m, e, 0, mesh.name)) return false;
        mesh.type = e.u16(0) == 1 ? 1 : 0;
        const uint8_t* p;
        size_t n;
        if (!get_prim_list(m, e, 1, 4, p, n)) return false;
        mesh.xyz.resize(n);
        if (n) std::memcpy(mesh.xyz.data(), p, 4 * n);
        s.meshes.push_back(std::move(mesh));
    }
    if (!get_struct_list(m, sc, 1, list)) return false;
    s.lights = (int32_t)list.size();
    if (!get_struct_list(m, sc, 2, list)) return false;
    for (const Struct& e : list) {
        mp_scene::Object o;
        Struct col;
        if (!get_text(m, e, 0, o.name) || !get_transform(m, e, 1, o.translation, o.rotation) ||
            !get_text(m, e, 2, o.meshname) || !get_struct(m, e, 3, col))
            return false;
        for (int k = 0; k < 3; ++k) o.color[k] = col.f32(k);
        s.objects.push_back(std::move(o));
    }
    if (!get_struct_list(m, sc, 3, list)) return false;
    for (const Struct& e : list) {
        mp_scene::Camera c;
        if (!get_text(m, e, 0, c.name) || !get_transform(m, e, 1, c.translation, c.rotation)) return false;
        c.near_plane = e.f32(0);
        c.far_plane = e.f32(1);
        c.fovy = e.f32(2);
        s.cameras.push_back(std::move(c));
    }
    // objects name their mesh (Scene.cpp:162-170, a map by name: the last
    // mesh of a name wins)
    for (auto& o : s.objects) {
        for (size_t k = 0; k < s.meshes.size(); ++k)
            if (s.meshes[k].name == o.meshname) o.mesh = (int32_t)k;
    }
    return true;
}

// ---------------------------------------------------------------------------
// transforms

// translate(mat4(1), t) * mat4_cast(quat(r, i, j, k)) (Scene.cpp:75-80), column
// major; the rotation from the unit quaternion by the standard formula.
void transform_matrix(const float t[3], const float q[4], float m[16]) {
    const float w = q[0], x = q[1], y = q[2], z = q[3];
    const float xx = x * x, yy = y * y, zz = z * z, xz = x * z, xy = x * y, yz = y * z;
    const float wx = w * x, wy = w * y, wz = w * z;
    std::memset(m, 0, 16 * sizeof(float));
    m[0] = 1.0f - 2.0f * (yy + zz);
    m[1] = 2.0f * (xy + wz);
    m[2] = 2.0f * (xz - wy);
    m[4] = 2.0f * (xy - wz);
    m[5] = 1.0f - 2.0f * (xx + zz);
    m[6] = 2.0f * (yz + wx);
    m[8] = 2.0f * (xz + wy);
    m[9] = 2.0f * (yz - wx);
    m[10] = 1.0f - 2.0f * (xx + yy);
    m[12] = t[0];
    m[13] = t[1];
    m[14] = t[2];
    m[15] = 1.0f;
}

// Inverse of a 4x4 column-major matrix by cofactors, in double, rounded once.
bool invert(const float a[16], float out[16]) {
    double m[16], inv[16];
    for (int i = 0; i < 16; ++i) m[i] = a[i];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] +
             m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
             m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] +
             m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
              m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
             m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] +
             m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
             m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
              m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] +
             m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] -
             m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] +
              m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
              m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] -
             m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] +
             m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] -
              m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] +
              m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0 || !std::isfinite(det)) return false;
    for (int i = 0; i < 16; ++i) out[i] = (float)(inv[i] / det);
    return true;
}

// a * b, column major, each element summed left to right in float.
void mul(const float a[16], const float b[16], float out[16]) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            float s = a[r] * b[4 * c];
            s = s + a[4 + r] * b[4 * c + 1];
            s = s + a[8 + r] * b[4 * c + 2];
            s = s + a[12 + r] * b[4 * c + 3];
            out[4 * c + r] = s;
        }
}

}  // namespace

extern "C" {

mp_status mp_scene_load(const char* path, mp_scene** out) {
    if (!path || !out) return MP_ERR_INVALID_ARG;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return MP_ERR_INVALID_ARG;
    std::vector<uint8_t> bytes;
    uint8_t buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + got);
    std::fclose(f);
    return mp_scene_parse(bytes.data(), bytes.size(), out);
}

mp_status mp_scene_parse(const uint8_t* data, size_t size, mp_scene** out) {
    if (!data || !out) return MP_ERR_INVALID_ARG;
    *out = nullptr;
    Message m;
    if (!unpack(data, size, m.w) || !parse_frame(m)) return MP_ERR_INVALID_ARG;
    static std::atomic<uint64_t> next_uid{1};
    mp_scene* s = new mp_scene();
    s->uid = next_uid.fetch_add(1);
    if (!decode(m, *s)) {
        delete s;
        return MP_ERR_INVALID_ARG;
    }
    *out = s;
    return MP_OK;
}

void mp_scene_free(mp_scene* s) { delete s; }

mp_status mp_scene_counts(const mp_scene* s, int32_t* meshes, int32_t* objects, int32_t* cameras, int32_t* lights) {
    if (!s) return MP_ERR_INVALID_ARG;
    if (meshes) *meshes = (int32_t)s->meshes.size();
    if (objects) *objects = (int32_t)s->objects.size();
    if (cameras) *cameras = (int32_t)s->cameras.size();
    if (lights) *lights = s->lights;
    return MP_OK;
}

mp_status mp_scene_mesh(const mp_scene* s, int32_t i, const char** name, int32_t* type, const float** xyz,
                        int64_t* n_floats) {
    if (!s || i < 0 || (size_t)i >= s->meshes.size()) return MP_ERR_INVALID_ARG;
    const auto& m = s->meshes[(size_t)i];
    if (name) *name = m.name.c_str();
    if (type) *type = m.type;
    if (xyz) *xyz = m.xyz.data();
    if (n_floats) *n_floats = (int64_t)m.xyz.size();
    return MP_OK;
}

mp_status mp_scene_object(const mp_scene* s, int32_t i, const char** name, int32_t* mesh, float matrix[16],
                          float color[4]) {
    if (!s || i < 0 || (size_t)i >= s->objects.size()) return MP_ERR_INVALID_ARG;
    const auto& o = s->objects[(size_t)i];
    if (name) *name = o.name.c_str();
    if (mesh) *mesh = o.mesh;
    if (matrix) transform_matrix(o.translation, o.rotation, matrix);
    if (color) {
        for (int k = 0; k < 3; ++k) color[k] = o.color[k];
        color[3] = 1.0f;   // vec4(color, 1) (Scene.cpp:166)
    }
    return MP_OK;
}

mp_status mp_scene_camera(const mp_scene* s, int32_t i, const char** name, float matrix[16], float* near_plane,
                          float* far_plane, float* fovy_deg) {
    if (!s || i < 0 || (size_t)i >= s->cameras.size()) return MP_ERR_INVALID_ARG;
    const auto& c = s->cameras[(size_t)i];
    if (name) *name = c.name.c_str();
    if (matrix) transform_matrix(c.translation, c.rotation, matrix);
    if (near_plane) *near_plane = c.near_plane;
    if (far_plane) *far_plane = c.far_plane;
    if (fovy_deg) *fovy_deg = c.fovy;
    return MP_OK;
}

mp_status mp_scene_modelview(const mp_scene* s, int32_t camera, int32_t object, float mv[16]) {
    if (!s || !mv || camera < 0 || (size_t)camera >= s->cameras.size() || object < 0 ||
        (size_t)object >= s->objects.size())
        return MP_ERR_INVALID_ARG;
    float cam[16], inv[16], obj[16];
    const auto& c = s->cameras[(size_t)camera];
    const auto& o = s->objects[(size_t)object];
    transform_matrix(c.translation, c.rotation, cam);
    transform_matrix(o.translation, o.rotation, obj);
    if (!invert(cam, inv)) return MP_ERR_INVALID_ARG;
    mul(inv, obj, mv);   // inverse(camera) * object (Scene.cpp:190)
    return MP_OK;
}

mp_status mp_scene_draw(mp_ctx* ctx, const mp_scene* s, int32_t camera) {
    if (!ctx || !s || camera < 0 || (size_t)camera >= s->cameras.size()) return MP_ERR_INVALID_ARG;
    int32_t window[2];
    mp_status st = mp_framebuffer(ctx, nullptr, nullptr, &window[0], &window[1], nullptr);
    if (st) return st;
    const auto& c = s->cameras[(size_t)camera];
    // Projection(fovy, near, window_size) (Scene.cpp:104-107)
    mp_projection proj;
    proj.fovy_deg = c.fovy;
    proj.near_plane = c.near_plane;
    proj.viewport[0] = window[0];
    proj.viewport[1] = window[1];
    if ((st = mp_prepare(ctx))) return st;
    for (size_t i = 0; i < s->objects.size(); ++i) {
        const auto& o = s->objects[i];
        if (o.mesh < 0) continue;   // an unknown mesh name draws nothing
        const auto& m = s->meshes[(size_t)o.mesh];
        // one handle per mesh, as the reference keys on Mesh* (Scene.cpp:186); built
        // from the scene's process-wide id rather than an address, so that a
        // later scene whose mesh lands at a freed one's address is loaded anew
        const uint64_t handle = (s->uid << 32) | (uint64_t)(uint32_t)o.mesh;
        int32_t loaded = 0;
        if ((st = mp_are_patches_loaded(ctx, handle, &loaded))) return st;
        if (!loaded && (st = mp_load_patches(ctx, handle, m.xyz.data(), m.xyz.size() / 3,
                                             m.type == 1 ? MP_GREGORY : MP_BEZIER)))
            return st;
        float mv[16], color[4];
        if ((st = mp_scene_modelview(s, camera, (int32_t)i, mv))) return st;
        mp_scene_object(s, (int32_t)i, nullptr, nullptr, nullptr, color);
        if ((st = mp_draw_patches(ctx, handle, mv, &proj, color))) return st;
    }
    return mp_finish(ctx);
}

}  // extern "C"
