// Pin driver: calls the reference's own src/base/Patch.cpp and
// src/base/Projection.cpp (compiled from the reference tree by build_ref.sh
// over the glm stand-in in refshim/) so the oracle's restated arithmetic can
// be compared with the reference's.  TEST INFRASTRUCTURE ONLY.
#include "Patch.h"
#include "Projection.h"
#include "ReyesConfig.h"

#include <vector>

ReyesConfigStandIn reyes_config;

extern "C" {

void refpin_eval_patch(const float* cp, float t, float s, float* out) {
    BezierPatch p;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            const float* q = cp + 3 * (4 * i + j);
            p.P[i][j] = vec3(q[0], q[1], q[2]);
        }
    vec3 r;
    eval_patch(p, t, s, r);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void refpin_eval_gregory(const float* cp, float u, float v, float* out) {
    vec3 pts[20];
    for (int k = 0; k < 20; ++k) pts[k] = vec3(cp[3 * k], cp[3 * k + 1], cp[3 * k + 2]);
    vec3 r;
    eval_gregory_patch(pts, u, v, r);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

int refpin_projection_bound(float fovy, float near_plane, int w, int h, float ribbon,
                            const float* box, float* size) {
    reyes_config.ribbon = ribbon;
    Reyes::Projection proj(fovy, near_plane, ivec2(w, h));
    BBox b;
    b.min = vec3(box[0], box[1], box[2]);
    b.max = vec3(box[3], box[4], box[5]);
    vec2 sz(0.0f, 0.0f);
    bool cull = false;
    proj.bound(b, sz, cull);
    size[0] = sz.x; size[1] = sz.y;
    return cull ? 1 : 0;
}

// Projection::calc_projection (src/base/Projection.cpp:37-40): the glm
// perspective matrix the reference's dice kernel gets, column major.
void refpin_projection_matrix(float fovy, float near_plane, int w, int h, float* out16) {
    Reyes::Projection projection(fovy, near_plane, ivec2(w, h));
    mat4 proj;
    projection.calc_projection(proj);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out16[4 * c + r] = proj[c][r];
}

// Projection::f() and the diagonal of Projection::calc_screen_matrix
// (src/base/Projection.cpp:47-50): what init_projection_buffer stores for the
// reference's GPU bound criterion besides the projection matrix.
void refpin_screen_params(float fovy, float near_plane, int w, int h, float* f2, float* vp2) {
    Reyes::Projection projection(fovy, near_plane, ivec2(w, h));
    mat2 sm;
    projection.calc_screen_matrix(sm);
    f2[0] = projection.f().x;
    f2[1] = projection.f().y;
    vp2[0] = sm[0][0];
    vp2[1] = sm[1][1];
}

// The LIFO loop of src/Reyes/BoundNSplitCLCPU.cpp:75-159 and the range bound
// of :249-336, written over the reference's eval_patch / eval_gregory_patch,
// BBox, maximum and Projection::bound.
long refpin_bound_n_split(const float* cp_in, int n_patches, int type, const float* mv16,
                          float fovy, float near_plane, int w, int h, float ribbon, float limit,
                          int max_split_depth, int* pid, float* range, long cap) {
    reyes_config.ribbon = ribbon;
    Reyes::Projection projection(fovy, near_plane, ivec2(w, h));
    mat4 mv;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) mv[c][r] = mv16[4 * c + r];
    int per = type == 0 ? 16 : 20;
    std::vector<vec3> patches((size_t)n_patches * per);
    for (size_t k = 0; k < patches.size(); ++k)
        patches[k] = vec3(cp_in[3 * k], cp_in[3 * k + 1], cp_in[3 * k + 2]);
    struct R { float x0, y0, x1, y1; size_t depth, id; };
    std::vector<R> stack((size_t)n_patches);
    for (int i = 0; i < n_patches; ++i) stack[(size_t)i] = R{0, 0, 1, 1, 0, (size_t)i};
    long n = 0;
    const size_t RES = 3;
    while (!stack.empty()) {
        R r = stack.back();
        stack.pop_back();
        vec3 ps[RES][RES];
        BBox box;
        box.clear();
        for (size_t iu = 0; iu < RES; ++iu)
            for (size_t iv = 0; iv < RES; ++iv) {
                float v = r.x0 + (r.x1 - r.x0) * iu * (1.0f / (RES - 1));
                float u = r.y0 + (r.y1 - r.y0) * iv * (1.0f / (RES - 1));
                vec3 pos;
                if (type == 0)
                    eval_patch(*((BezierPatch*)&patches[16 * r.id]), u, v, pos);
                else
                    eval_gregory_patch(&patches[20 * r.id], u, v, pos);
                vec3 pt = vec3(mv * vec4(pos, 1));
                box.add_point(pt);
                ps[iu][iv] = pt;
            }
        float vlen = 0, hlen = 0;
        for (size_t i = 0; i < RES; ++i) {
            float hh = 0, vv = 0;
            for (size_t j = 0; j < RES - 1; ++j) {
                vv += glm::distance(ps[j][i], ps[j + 1][i]);
                hh += glm::distance(ps[i][j], ps[i][j + 1]);
            }
            vlen = maximum(vv, vlen);
            hlen = maximum(hh, hlen);
        }
        vec2 size;
        bool cull;
        projection.bound(box, size, cull);
        if (cull) continue;
        if (box.min.z < 0 && size.x < limit && size.y < limit) {
            if (n < cap) {
                pid[n] = (int)r.id;
                range[4 * n] = r.x0; range[4 * n + 1] = r.y0;
                range[4 * n + 2] = r.x1; range[4 * n + 3] = r.y1;
            }
            ++n;
        } else if (r.depth > (size_t)max_split_depth) {
        } else if (vlen < hlen) {
            float cy = (r.y0 + r.y1) * 0.5f;
            stack.push_back(R{r.x0, r.y0, r.x1, cy, r.depth + 1, r.id});
            stack.push_back(R{r.x0, cy, r.x1, r.y1, r.depth + 1, r.id});
        } else {
            float cx = (r.x0 + r.x1) * 0.5f;
            stack.push_back(R{r.x0, r.y0, cx, r.y1, r.depth + 1, r.id});
            stack.push_back(R{cx, r.y0, r.x1, r.y1, r.depth + 1, r.id});
        }
    }
    return n;
}
}
