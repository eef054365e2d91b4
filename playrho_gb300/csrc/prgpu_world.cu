// prgpu_world.cu -- host side of the C ABI: batch creation (mass data, proxies,
// device allocation), step orchestration with CUDA-graph replay, queries.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>
#include <mutex>

#include "../../include/prgpu.h"
#include "prgpu_kernels.cuh"

using namespace prgpu;

// Sizes of a batch's device arrays.
struct WorldDims {
    uint32_t W, N, S, J, C, K, V, JO, JC;  // worlds, bodies, shapes, joints, contact and candidate
                                           // capacity, vertices, joint-partner and collide entries
};

struct prgpu_world {
    int device = 0;
    cudaStream_t stream = nullptr;
    DW d{};
    Launch L{};
    std::vector<void*> allocs;
    std::vector<size_t> alloc_bytes;
    std::vector<bool> alloc_scratch;  // rewritten every step before it is read: not checkpointed
    cudaGraphExec_t graph = nullptr;
    cudaGraph_t graph_def = nullptr;
    prgpu_step_conf conf{};
    bool conf_valid = false;
    std::string err;
    DConf* d_conf = nullptr;
    float* d_stage = nullptr;
    uint32_t* d_stage_u = nullptr;
    Counters* h_cnt = nullptr;  // pinned mirror of the device counters
    // pinned copy of the device error word and site, written by every graph-replayed
    // step as it ends (read by prgpu_step_async without waiting)
    uint32_t* h_err = nullptr;
    WorldDims dims{};            // sizes the device arrays were allocated with
    bool grow = false;           // prgpu_set_capacity_growth
    void* backup = nullptr;      // the state before the step in flight (growth on)
    size_t backup_bytes = 0;
    float4* post_imp = nullptr;  // solve records (prgpu_set_solve_records), allocated on first use
    uint2* post_tag = nullptr;
    bool stepped = false;       // a step has run: proxies exist
    cudaEvent_t graph_ev[8] = {};  // recorded by the captured step between its phases
    std::vector<uint32_t> order_nb;  // body counts of the worlds in work-queue order
    struct AdjWindow* adj = nullptr;  // open StepAdjoint window, if any
    uint32_t warp_world_max = 0;     // worlds of at most this many bodies are swept by one warp,
    uint32_t group_world_max = 0;    //   of at most this many (if larger) by a group of 64 threads
    // time-of-impact phase: set-up, one round, and the final update, each captured once
    cudaGraphExec_t toi_graph[3] = {};
};

extern "C" void adjoint_drop_graphs(prgpu_world* w);

extern "C" {
static int alloc_world(prgpu_world* w, const WorldDims& z);
static int snap_copy(prgpu_world* w, void* buf, bool save);
static size_t snap_size(const prgpu_world* w);
}

namespace {

int fail(prgpu_world* w, int code, const char* fmt, ...) {
    if (w) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        w->err = buf;
    }
    return code;
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        const cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return fail(w, PRGPU_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int dalloc(prgpu_world* w, T** p, size_t n, bool scratch = false) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    const cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return fail(w, PRGPU_ECUDA, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    w->allocs.push_back(q);
    w->alloc_bytes.push_back(bytes);
    w->alloc_scratch.push_back(scratch);
    *p = static_cast<T*>(q);
    return PRGPU_OK;
}

// ---- host restatement of the mass-data computation (MassData.cpp, WorldBody.cpp) ----
struct HV {
    float x, y;
};
inline HV hv(float x, float y) { return HV{x, y}; }
inline HV operator+(HV a, HV b) { return hv(a.x + b.x, a.y + b.y); }
inline HV operator-(HV a, HV b) { return hv(a.x - b.x, a.y - b.y); }
inline HV hmul(HV a, float s) { return hv(a.x * s, a.y * s); }
inline HV hdiv(HV a, float s) { const float inv = 1.0f / s; return hv(a.x * inv, a.y * inv); }
inline float hcross(HV a, HV b) { const float m = a.x * b.y; const float s = a.y * b.x; return m - s; }
inline float hmag2(HV a) { float r = 0.f; r += a.x * a.x; r += a.y * a.y; return r; }
inline HV hrevperp(HV a) { return hv(-a.y, a.x); }
inline HV hfwdperp(HV a) { return hv(a.y, -a.x); }
inline HV hunit(HV v, HV fb) {
    const float m2 = v.x * v.x + v.y * v.y;
    if (std::isnormal(m2)) {
        const float m = std::sqrt(m2);
        const float inv = 1.0f / m;
        return hv(v.x * inv, v.y * inv);
    }
    const float m = std::hypot(v.x, v.y);
    if (!std::isnormal(m)) return fb;
    return hv(v.x / m, v.y / m);
}
inline HV hrotate(HV v, HV q) { return hv((q.x * v.x) - (q.y * v.y), (q.y * v.x) + (q.x * v.y)); }

void shape_mass(int nv, const HV* v, float r, float density, float& mass, HV& center, float& I) {
    const float Pi = 3.14159265358979323846264338327950288f;
    if (nv == 1) {
        const float r2 = r * r;
        const float area = r2 * Pi;
        mass = density * area;
        const float Iz = area * ((r2 / 2.0f) + hmag2(v[0]));
        I = Iz * density;
        center = v[0];
        return;
    }
    if (nv == 2) {
        const float r2 = r * r;
        const float circle_area = r2 * Pi;
        const float circle_mass = density * circle_area;
        const HV v0 = v[0], v1 = v[1];
        const HV dd = v1 - v0;
        const HV offset = hmul(hrevperp(hunit(dd, hv(0.f, 0.f))), r);
        const float b = std::sqrt(hmag2(dd));
        const float h = r * 2.0f;
        const float rect_mass = density * b * h;
        mass = circle_mass + rect_mass;
        center = hdiv(v0 + v1, 2.0f);
        const float halfCircleArea = circle_area / 2.0f;
        const float halfRSquared = r2 / 2.0f;
        const HV q[4] = {v0 + offset, v0 - offset, v1 - offset, v1 + offset};
        float sum_x = 0.f, sum_y = 0.f;
        for (int i = 0; i < 4; ++i) {
            const HV tv = q[i], nx = q[(i + 1) % 4];
            const float fb = hcross(tv, nx);
            sum_x += ((tv.y * tv.y) + tv.y * nx.y + (nx.y * nx.y)) * fb;
            sum_y += ((tv.x * tv.x) + tv.x * nx.x + (nx.x * nx.x)) * fb;
        }
        const float Iz = (sum_x + sum_y) * (1.0f / 12.0f);
        const float I0 = halfCircleArea * (halfRSquared + hmag2(v0));
        const float I1 = halfCircleArea * (halfRSquared + hmag2(v1));
        I = (I0 + I1 + Iz) * density;
        return;
    }
    HV ctr = hv(0.f, 0.f);
    float area = 0.f, II = 0.f;
    HV s0 = hv(0.f, 0.f);
    for (int i = 0; i < nv; ++i) s0 = s0 + v[i];
    s0 = hdiv(s0, (float)nv);
    for (int i = 0; i < nv; ++i) {
        const HV e1 = v[i] - s0;
        const HV e2 = v[(i + 1) % nv] - s0;
        const float D = hcross(e1, e2);
        const float triangleArea = D * (1.0f / 2.0f);
        area += triangleArea;
        ctr = ctr + hmul(hmul(e1 + e2, triangleArea), 1.0f / 3.0f);
        const float intx2 = (e1.x * e1.x) + e2.x * e1.x + (e2.x * e2.x);
        const float inty2 = (e1.y * e1.y) + e2.y * e1.y + (e2.y * e2.y);
        II += D * (intx2 + inty2) * (1.0f / 12.0f);
    }
    const float m = density * area;
    ctr = ((area > 0.f) && !(std::fabs(area) < 1.17549435e-38f)) ? hdiv(ctr, area) : hv(0.f, 0.f);
    const HV mdc = ctr + s0;
    const float inertialLever = hmag2(mdc) - hmag2(ctr);
    mass = m;
    center = mdc;
    I = (density * II) + (m * inertialLever);
}

struct HostBody {
    int type;
    uint32_t flags;
    float px, py, a;  // pos1 (centre)
    float vx, vy, w;
    float lcx, lcy;
    float xpx, xpy, xc, xs;  // cached transformation
    float invM, invI;
};

void host_set_pos(HostBody& b, float px, float py, float a) {
    b.px = px; b.py = py; b.a = a;
    const float c = std::cos(a), s = std::sin(a);
    const HV p = hv(px, py) - hrotate(hv(b.lcx, b.lcy), hv(c, s));
    b.xpx = p.x; b.xpy = p.y; b.xc = c; b.xs = s;
}

// GetMassData of a multi-child shape from its consecutive children
// shapes[k0 .. k0+n-1]: ChainShapeConf (edges; ChainShapeConf.cpp:113-147: summed
// masses, inertias and mass-weighted centres, the centre divided by the summed
// segment areas) or MultiShapeConf (hulls; MultiShapeConf.cpp:35-57: the centre
// divided by the mass).
void group_mass(const std::vector<int>& shapes, size_t k0, size_t n, bool chain, const prgpu_batch_desc* ds,
                const std::vector<std::vector<HV>>& sv, float& mass, HV& center, float& I) {
    const float Pi = 3.14159265358979323846f;
    float m = 0.f, iz = 0.f, area = 0.f;
    HV c = hv(0.f, 0.f);
    for (size_t k = k0; k < k0 + n; ++k) {
        const int s = shapes[k];
        float mk, ik;
        HV ck;
        shape_mass((int)sv[s].size(), sv[s].data(), ds->shape_radius[s], ds->shape_density[s], mk, ck, ik);
        m += mk;
        iz += ik;
        c = c + hmul(ck, mk);
        if (chain) {
            const HV d = sv[s][1] - sv[s][0];
            const float bl = std::sqrt(hmag2(d));
            const float r = ds->shape_radius[s];
            const float h = r * 2.0f;
            area += bl * h + (r * r) * Pi;
        }
    }
    if (chain) c = hdiv(c, area);
    else c = (m > 0.f) ? hdiv(c, m) : hv(0.f, 0.f);
    mass = m; center = c; I = iz;
}

// ResetMassData -> ComputeMassData -> SetMassData over the shapes attached so far.
void reset_mass(HostBody& b, const std::vector<int>& shapes, const prgpu_batch_desc* ds,
                const std::vector<std::vector<HV>>& sv) {
    float mass = 0.f, I = 0.f;
    HV wc = hv(0.f, 0.f);
    for (size_t k = 0; k < shapes.size(); ++k) {
        const int s = shapes[k];
        const int own = ds->shape_owner ? ds->shape_owner[s] : -1;
        if (own >= 0 && own != s) continue;  // a later child: counted with the first
        if (ds->shape_density[s] > 0.f) {
            float m, i;
            HV c;
            if (own == s) {
                size_t n = 1;
                while (k + n < shapes.size() && ds->shape_owner[shapes[k + n]] == s) ++n;
                group_mass(shapes, k, n, ds->shape_kind[s] == PRGPU_EDGE, ds, sv, m, c, i);
            } else {
                shape_mass((int)sv[s].size(), sv[s].data(), ds->shape_radius[s], ds->shape_density[s], m, c, i);
            }
            mass += m;
            wc = wc + hmul(c, m);
            I += i;
        }
    }
    const HV center = (mass > 0.f) ? hdiv(wc, mass) : hv(0.f, 0.f);
    if (b.type != PRGPU_DYNAMIC) {
        b.invM = 0.f; b.invI = 0.f;
        if (b.type == PRGPU_STATIC) {
            const float lx = b.xpx, ly = b.xpy, a = b.a;
            b.lcx = 0.f; b.lcy = 0.f;
            host_set_pos(b, lx, ly, a);
        }
        return;
    }
    const float m = (mass > 0.f) ? mass : 1.0f;
    b.invM = 1.0f / m;
    b.invI = 0.f;
    if ((I > 0.f) && !(b.flags & PRGPU_BODY_FIXED_ROTATION)) {
        const float Ic = I - (m * hmag2(center));
        b.invI = 1.0f / Ic;
    }
    const HV oldCenter = hv(b.px, b.py);
    const HV np = hrotate(center, hv(b.xc, b.xs)) + hv(b.xpx, b.xpy);
    b.lcx = center.x; b.lcy = center.y;
    host_set_pos(b, np.x, np.y, b.a);
    const HV dc = hv(b.px, b.py) - oldCenter;
    const HV dv = hmul(hrevperp(dc), b.w);
    b.vx = b.vx + dv.x; b.vy = b.vy + dv.y;
}

struct HostPrep {
    uint32_t W = 0, N = 0, S = 0, J = 0, V = 0;
    std::vector<uint32_t> body_off, shape_off, joint_off, body_world;
    std::vector<std::vector<HV>> sv;
    std::vector<std::vector<int>> body_shapes;
    std::vector<HostBody> hb;
    std::vector<float4> pos1, vel, mass, acc, xfh;
    std::vector<float2> damp;
    std::vector<uint32_t> bflags;
    std::vector<uint32_t> s_meta, s_voff, s_filter, s_body, p_state;
    std::vector<int32_t> s_group;
    std::vector<float> s_radius;
    std::vector<float2> s_mat;
    std::vector<float4> vtx;
    std::vector<uint32_t> jcnt, joff, jother, jcc, jcur;
    std::vector<float4> j_anchor, j_param, j_zero, j_extra, j_gear;
    std::vector<float> j_maxtorque;
    std::vector<uint32_t> j_bodies, j_flags;
};

// Validation and host-side preparation of a batch: flattening, mass data
// (Attach with resetMassData after each shape), normals, joint lists.
int prepare_host(const prgpu_batch_desc* ds, HostPrep& hp) {
    const uint32_t W = ds->n_worlds, N = ds->n_bodies, S = ds->n_shapes, J = ds->n_joints, V = ds->n_verts;
    hp.W = W; hp.N = N; hp.S = S; hp.J = J; hp.V = V;
    if (W == 0) return PRGPU_EINVAL;
    // ---- validate and flatten
    auto& body_off = hp.body_off; auto& shape_off = hp.shape_off; auto& joint_off = hp.joint_off;
    body_off.assign(W + 1, 0); shape_off.assign(W + 1, 0); joint_off.assign(W + 1, 0);
    for (uint32_t k = 0; k < W; ++k) {
        body_off[k + 1] = body_off[k] + ds->world_body_count[k];
        shape_off[k + 1] = shape_off[k] + ds->world_shape_count[k];
        joint_off[k + 1] = joint_off[k] + (ds->world_joint_count ? ds->world_joint_count[k] : 0u);
    }
    if (body_off[W] != N || shape_off[W] != S || joint_off[W] != J) return PRGPU_EINVAL;
    auto& body_world = hp.body_world; body_world.assign(N, 0);
    for (uint32_t k = 0; k < W; ++k)
        for (uint32_t b = body_off[k]; b < body_off[k + 1]; ++b) body_world[b] = k;
    auto& sv = hp.sv; sv.assign(S, {});
    auto& body_shapes = hp.body_shapes; body_shapes.assign(N, {});
    for (uint32_t s = 0; s < S; ++s) {
        const uint32_t b = ds->shape_body[s];
        const uint32_t nv = ds->shape_nv[s];
        if (b >= N || nv < 1 || nv > 16u || ds->shape_voff[s] + nv > V) return PRGPU_EINVAL;
        const int kind = ds->shape_kind[s];
        // A polygon whose points de-duplicate to one or two vertices stays valid
        // (PolygonShapeConf::Set keeps what VertexSet leaves); collision dispatches
        // on the vertex count.
        if ((kind == PRGPU_DISK && nv != 1) || (kind == PRGPU_EDGE && nv != 2) || kind < 0 || kind > 2)
            return PRGPU_EINVAL;
        for (uint32_t i = 0; i < nv; ++i)
            sv[s].push_back(hv(ds->verts[2 * (ds->shape_voff[s] + i)], ds->verts[2 * (ds->shape_voff[s] + i) + 1]));
    }
    for (uint32_t k = 0; k < W; ++k) {
        for (uint32_t s = shape_off[k]; s < shape_off[k + 1]; ++s) {
            const uint32_t b = ds->shape_body[s];
            if (b < body_off[k] || b >= body_off[k + 1]) return PRGPU_EINVAL;
        }
    }
    // ---- bodies: BodyConf -> Body, then Attach(..., resetMassData = true) per shape
    auto& hb = hp.hb; hb.assign(N, HostBody{});
    for (uint32_t b = 0; b < N; ++b) {
        HostBody& x = hb[b];
        x.type = ds->body_type[b];
        if (x.type < 0 || x.type > 2) return PRGPU_EINVAL;
        x.flags = ds->body_flags[b];
        x.lcx = x.lcy = 0.f;
        host_set_pos(x, ds->body_pos[3 * b], ds->body_pos[3 * b + 1], ds->body_pos[3 * b + 2]);
        if (x.type == PRGPU_STATIC) { x.vx = x.vy = x.w = 0.f; }
        else { x.vx = ds->body_vel[3 * b]; x.vy = ds->body_vel[3 * b + 1]; x.w = ds->body_vel[3 * b + 2]; }
        x.invM = (x.type == PRGPU_DYNAMIC) ? 1.0f : 0.0f;
        x.invI = 0.f;
    }
    for (uint32_t s = 0; s < S; ++s) {
        const uint32_t b = ds->shape_body[s];
        body_shapes[b].push_back((int)s);
        // Attach(..., resetMassData = true) once per shape of the reference: after
        // the last child of a multi-child shape
        const int own = ds->shape_owner ? ds->shape_owner[s] : -1;
        if (own >= 0) {
            const bool first = own == (int)s;
            if (own > (int)s || ds->shape_body[own] != b || ds->shape_owner[own] != own ||
                (!first && ds->shape_owner[s - 1] != own) || ds->shape_kind[s] != ds->shape_kind[own] ||
                (ds->shape_kind[s] == PRGPU_DISK))
                return PRGPU_EINVAL;
        }
        const bool last = own < 0 || s + 1 == S || ds->shape_owner[s + 1] != own;
        if (last) reset_mass(hb[b], body_shapes[b], ds, sv);
    }
    if (ds->body_mass) {
        // SetMassData (Body.cpp): the transformation stays, the centre moves to
        // the given local centre; only dynamic bodies take a mass.
        for (uint32_t b = 0; b < N; ++b) {
            HostBody& x = hb[b];
            if (x.type != PRGPU_DYNAMIC) continue;
            const float* m = ds->body_mass + 4 * b;
            if (!(m[0] >= 0.f) || !(m[1] >= 0.f)) return PRGPU_EINVAL;
            x.invM = m[0]; x.invI = m[1]; x.lcx = m[2]; x.lcy = m[3];
            const HV c = hv(x.xpx, x.xpy) + hrotate(hv(x.lcx, x.lcy), hv(x.xc, x.xs));
            x.px = c.x; x.py = c.y;
        }
    }
    // ---- host arrays in device layout
    auto& pos1 = hp.pos1; auto& vel = hp.vel; auto& mass = hp.mass; auto& acc = hp.acc;
    pos1.resize(N); vel.resize(N); mass.resize(N); acc.resize(N);
    auto& damp = hp.damp; damp.resize(N);
    auto& bflags = hp.bflags; bflags.resize(N);
    for (uint32_t b = 0; b < N; ++b) {
        const HostBody& x = hb[b];
        pos1[b] = make_float4(x.px, x.py, x.a, 0.f);
        vel[b] = make_float4(x.vx, x.vy, x.w, 0.f);
        mass[b] = make_float4(x.invM, x.invI, x.lcx, x.lcy);
        if (x.type == PRGPU_DYNAMIC) acc[b] = make_float4(ds->body_acc[3 * b], ds->body_acc[3 * b + 1], ds->body_acc[3 * b + 2], 0.f);
        else acc[b] = make_float4(0.f, 0.f, 0.f, 0.f);
        damp[b] = make_float2(ds->body_damp[2 * b], ds->body_damp[2 * b + 1]);
        uint32_t f = (uint32_t)x.type;
        if ((x.flags & PRGPU_BODY_AWAKE) && x.type != PRGPU_STATIC) f |= BF_AWAKE;
        if (x.flags & PRGPU_BODY_ALLOW_SLEEP) f |= BF_ALLOW_SLEEP;
        if (x.flags & PRGPU_BODY_FIXED_ROTATION) f |= BF_FIXED_ROT;
        if (x.flags & PRGPU_BODY_ENABLED) f |= BF_ENABLED;
        if (x.flags & PRGPU_BODY_BULLET) f |= BF_BULLET;
        bflags[b] = f;
    }
    auto& s_meta = hp.s_meta; auto& s_voff = hp.s_voff; auto& s_filter = hp.s_filter; auto& s_body = hp.s_body;
    auto& p_state = hp.p_state;
    s_meta.resize(S); s_voff.resize(S); s_filter.resize(S); s_body.resize(S); p_state.assign(S, 2u);
    auto& s_group = hp.s_group; s_group.resize(S);
    auto& s_radius = hp.s_radius; s_radius.resize(S);
    auto& s_mat = hp.s_mat; s_mat.resize(S);
    auto& vtx = hp.vtx; vtx.clear();
    vtx.reserve(V);
    for (uint32_t s = 0; s < S; ++s) {
        const int nv = (int)sv[s].size();
        // CreateBody / Attach queue a proxy only for a shape of an enabled body
        // (AabbTreeWorld.cpp:1040, :1302): the shapes of a disabled body get none.
        const bool no_proxy = !(hb[ds->shape_body[s]].flags & PRGPU_BODY_ENABLED);
        s_meta[s] = (uint32_t)ds->shape_kind[s] | ((uint32_t)nv << 8) | (ds->shape_filter[4 * s + 3] ? kShapeSensor : 0u) |
                    (no_proxy ? kShapeNoProxy : 0u);
        s_voff[s] = (uint32_t)vtx.size();
        // GetFwdNormalsVector (d2/Math.cpp)
        for (int i = 0; i < nv; ++i) {
            HV n = hv(0.f, 0.f);
            if (nv > 1) n = hunit(hfwdperp(sv[s][(i + 1) % nv] - sv[s][i]), hv(0.f, 0.f));
            vtx.push_back(make_float4(sv[s][i].x, sv[s][i].y, n.x, n.y));
        }
        s_radius[s] = ds->shape_radius[s];
        s_mat[s] = make_float2(ds->shape_friction[s], ds->shape_restitution[s]);
        s_filter[s] = ((uint32_t)ds->shape_filter[4 * s] & 0xffffu) | (((uint32_t)ds->shape_filter[4 * s + 1] & 0xffffu) << 16);
        s_group[s] = (int32_t)(int16_t)ds->shape_filter[4 * s + 2];
        s_body[s] = ds->shape_body[s];
    }
    // body -> joint CSR for ShouldCollide
    auto& jcnt = hp.jcnt; jcnt.assign(N + 1, 0);
    for (uint32_t j = 0; j < J; ++j) {
        const uint32_t a = ds->joint_bodies[2 * j], b = ds->joint_bodies[2 * j + 1];
        if (a >= N || b >= N) return PRGPU_EINVAL;
        jcnt[a]++;
        if (b != a) jcnt[b]++;
    }
    auto& joff = hp.joff; joff.assign(N + 1, 0);
    for (uint32_t b = 0; b < N; ++b) joff[b + 1] = joff[b] + jcnt[b];
    auto& jother = hp.jother; auto& jcc = hp.jcc; auto& jcur = hp.jcur;
    jother.assign(std::max<uint32_t>(joff[N], 1), 0); jcc.assign(std::max<uint32_t>(joff[N], 1), 0);
    jcur.assign(joff.begin(), joff.end() - 1);
    auto& j_anchor = hp.j_anchor; auto& j_param = hp.j_param; auto& j_zero = hp.j_zero;
    j_anchor.resize(J); j_param.resize(J); j_zero.assign(J, make_float4(0.f, 0.f, 0.f, 0.f));
    auto& j_maxtorque = hp.j_maxtorque; j_maxtorque.resize(J);
    auto& j_bodies = hp.j_bodies; auto& j_flags = hp.j_flags; j_bodies.resize(2 * J); j_flags.resize(J);
    hp.j_extra.assign(2 * (size_t)J, make_float4(0.f, 0.f, 0.f, 0.f));
    for (uint32_t j = 0; j < J; ++j) {
        const uint32_t a = ds->joint_bodies[2 * j], b = ds->joint_bodies[2 * j + 1];
        const uint32_t cc = ds->joint_flags[3 * j + 2] ? 1u : 0u;
        jother[jcur[a]] = b; jcc[jcur[a]++] = cc;
        if (b != a) { jother[jcur[b]] = a; jcc[jcur[b]++] = cc; }
        j_bodies[2 * j] = a; j_bodies[2 * j + 1] = b;
        j_anchor[j] = make_float4(ds->joint_anchors[4 * j], ds->joint_anchors[4 * j + 1], ds->joint_anchors[4 * j + 2], ds->joint_anchors[4 * j + 3]);
        j_param[j] = make_float4(ds->joint_params[6 * j], ds->joint_params[6 * j + 1], ds->joint_params[6 * j + 2], ds->joint_params[6 * j + 3]);
        j_maxtorque[j] = ds->joint_params[6 * j + 4];
        const int32_t kind = ds->joint_type ? ds->joint_type[j] : PRGPU_JOINT_REVOLUTE;
        if (kind < PRGPU_JOINT_REVOLUTE || kind > PRGPU_JOINT_GEAR) return PRGPU_EINVAL;
        if (kind == PRGPU_JOINT_TARGET && a != b) return PRGPU_EINVAL;
        j_flags[j] = (ds->joint_flags[3 * j] ? 1u : 0u) | (ds->joint_flags[3 * j + 1] ? 2u : 0u) | (cc << 2) |
                     ((uint32_t)kind << 8);
        const float* e = ds->joint_extra ? ds->joint_extra + 8 * (size_t)j : nullptr;
        hp.j_extra[2 * j] = e ? make_float4(e[0], e[1], e[2], e[3]) : make_float4(0.f, 0.f, 0.f, 0.f);
        hp.j_extra[2 * j + 1] = e ? make_float4(e[4], e[5], e[6], e[7]) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (kind == PRGPU_JOINT_PRISMATIC || kind == PRGPU_JOINT_WHEEL) {
            // localXAxisA = UnitVec::Get(axis) (UnitVec.hpp:175-235)
            const V2 ax = unit_vector(mk(hp.j_extra[2 * j].x, hp.j_extra[2 * j].y), mk(0.f, 0.f));
            hp.j_extra[2 * j].x = ax.x; hp.j_extra[2 * j].y = ax.y;
        }
    }
    // Gear joints: GetGearJointConf(world, joint1, joint2, ratio) (GearJointConf.cpp:
    // 66-160) on the bodies' state at creation; joint_extra = joint1 joint2 ratio
    // (global indices of two earlier revolute or prismatic joints of the same world).
    hp.j_gear.assign(5 * (size_t)J, make_float4(0.f, 0.f, 0.f, 0.f));
    auto body_angle = [&](uint32_t b) { return ds->body_pos[3 * b + 2]; };
    auto body_xf = [&](uint32_t b) {
        const float an = ds->body_pos[3 * b + 2];
        return Xf{mk(ds->body_pos[3 * b], ds->body_pos[3 * b + 1]), mk(std::cos(an), std::sin(an))};
    };
    auto bits = [](uint32_t u) { float f; std::memcpy(&f, &u, sizeof f); return f; };
    for (uint32_t j = 0; j < J; ++j) {
        if (!ds->joint_type || ds->joint_type[j] != PRGPU_JOINT_GEAR) continue;
        const float* e = ds->joint_extra ? ds->joint_extra + 8 * (size_t)j : nullptr;
        if (!e) return PRGPU_EINVAL;
        const float f1 = e[0], f2 = e[1], ratio = e[2];
        if (!(f1 >= 0.f && f2 >= 0.f && f1 < (float)j && f2 < (float)j) || f1 != std::floor(f1) || f2 != std::floor(f2))
            return PRGPU_EINVAL;
        const uint32_t j1 = (uint32_t)f1, j2 = (uint32_t)f2;
        const int32_t k1 = ds->joint_type[j1], k2 = ds->joint_type[j2];
        if ((k1 != PRGPU_JOINT_REVOLUTE && k1 != PRGPU_JOINT_PRISMATIC) ||
            (k2 != PRGPU_JOINT_REVOLUTE && k2 != PRGPU_JOINT_PRISMATIC))
            return PRGPU_EINVAL;
        const uint32_t A = ds->joint_bodies[2 * j1 + 1], B = ds->joint_bodies[2 * j2 + 1];
        const uint32_t C = ds->joint_bodies[2 * j1], D = ds->joint_bodies[2 * j2];
        if (ds->joint_bodies[2 * j] != A || ds->joint_bodies[2 * j + 1] != B) return PRGPU_EINVAL;
        // the coordinate of body X against body Y through joint jj (its data out)
        auto coupling = [&](uint32_t jj, uint32_t X, uint32_t Y, float& ref, V2& la, V2& lb, V2& ax) -> float {
            if (ds->joint_type[jj] == PRGPU_JOINT_PRISMATIC) {
                la = mk(ds->joint_anchors[4 * jj], ds->joint_anchors[4 * jj + 1]);
                lb = mk(ds->joint_anchors[4 * jj + 2], ds->joint_anchors[4 * jj + 3]);
                ax = mk(hp.j_extra[2 * jj].x, hp.j_extra[2 * jj].y);
                const Xf xX = body_xf(X), xY = body_xf(Y);
                const V2 pX = invrotate(rotate(lb, xX.q) + (xX.p - xY.p), xY.q);
                return dot(pX - la, ax);
            }
            ref = ds->joint_params[6 * jj];
            return (body_angle(X) - body_angle(Y)) - ref;
        };
        float refAC = 0.f, refBD = 0.f;
        V2 laAC = mk(0.f, 0.f), lbAC = laAC, axAC = laAC, laBD = laAC, lbBD = laAC, axBD = laAC;
        const float scalar1 = coupling(j1, A, C, refAC, laAC, lbAC, axAC);
        const float scalar2 = coupling(j2, B, D, refBD, laBD, lbBD, axBD);
        // e[4] != 0: the caller's constant (a GearJointConf made earlier) instead
        const float constant = (e[4] != 0.f) ? e[3] : scalar1 + ratio * scalar2;
        float4* g = &hp.j_gear[5 * (size_t)j];
        g[0] = make_float4(bits(C), bits(D), bits(k1 == PRGPU_JOINT_PRISMATIC ? 1u : 0u),
                           bits(k2 == PRGPU_JOINT_PRISMATIC ? 1u : 0u));
        g[1] = make_float4(ratio, constant, refAC, refBD);
        g[2] = make_float4(laAC.x, laAC.y, lbAC.x, lbAC.y);
        g[3] = make_float4(axAC.x, axAC.y, laBD.x, laBD.y);
        g[4] = make_float4(lbBD.x, lbBD.y, axBD.x, axBD.y);
    }
    return PRGPU_OK;
}

int bits_for(uint64_t n) {
    int b = 1;
    while ((1ull << b) < n) ++b;
    return b;
}

// Phases of one step; `ev` (kPhases + 1 events) brackets them when profiling.
constexpr int kPhases = 7;
// Batches of at least this many worlds sweep one world per CTA by default.
constexpr uint32_t kPerWorldMinWorlds = 64;
// Shared memory of the per-world solver for staging body state (44 bytes a
// body; a warp gets an eighth).  0 by default: staging costs CTAs per SM, and
// the sweeps are bound by latency that staging does not remove; the autotuner
// tries it.
constexpr uint32_t kStageBytes = 0u;
constexpr uint32_t kStageChoices[] = {0u, 1024u * 44u, 2048u * 44u};
// Worlds of at most this many bodies are swept by one warp by default.
constexpr uint32_t kWarpWorldMaxBodies = 256;

// Queue entries of worlds above max_bodies (the queue is by decreasing size).
uint32_t count_worlds_above(const prgpu_world* w, uint32_t max_bodies) {
    uint32_t n = 0;
    while (n < w->order_nb.size() && w->order_nb[n] > max_bodies) ++n;
    return n;
}

void count_world_classes(prgpu_world* w) {
    w->d.n_world_mid = count_worlds_above(w, w->warp_world_max);
    w->d.n_world_big = count_worlds_above(w, std::max(w->warp_world_max, w->group_world_max));
}

uint32_t count_big_worlds(const prgpu_world* w) {
    uint32_t n = 0;
    while (n < w->order_nb.size() && w->order_nb[n] > w->warp_world_max) ++n;
    return n;
}

// Drops the captured step so that the next step captures the new launches.
int drop_graph(prgpu_world* w) {
    CU(cudaSetDevice(w->device));
    CU(cudaStreamSynchronize(w->stream));
    adjoint_drop_graphs(w);
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->graph_def) { cudaGraphDestroy(w->graph_def); w->graph_def = nullptr; }
    for (auto& g : w->toi_graph)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    return PRGPU_OK;
}

int enqueue_step(prgpu_world* w, bool solve, cudaEvent_t* ev = nullptr, bool capturing = false) {
    const DW& d = w->d;
    const Launch& L = w->L;
    cudaStream_t s = w->stream;
    // Inside a capture only external records become event nodes of the graph.
    auto mark = [&](int k) {
        if (!ev) return;
        if (capturing) cudaEventRecordWithFlags(ev[k], s, cudaEventRecordExternal);
        else cudaEventRecord(ev[k], s);
    };
    mark(0);
    launch_reset_step(d, L, s);
    // pre-phase (AabbTreeWorld.cpp:2159-2199)
    launch_pre_proxies(d, L, s);
    launch_destroy_contacts(d, L, s);
    launch_update_contacts(d, L, BF_DIRTY, s);
    launch_find_contacts(d, L, s);
    mark(1);
    if (solve) {
        launch_islands_colour(d, L, s);
        mark(2);
        launch_build_constraints(d, L, s);
        mark(3);
        launch_solve_sweeps(d, L, s);
        mark(4);
        launch_solve_finish(d, L, s);
        if (d.cs_post_tag) launch_post_record(d, L, s);
        mark(5);
        // post-solve contact maintenance (AabbTreeWorld.cpp:1532-1557)
        launch_set_upd_phase(d, kUpdPost, s);
        launch_synchronize(d, L, s);
        launch_update_contacts(d, L, BF_MOVED, s);
        mark(6);
        launch_find_contacts(d, L, s);
    } else {
        for (int k = 2; k <= 6; ++k) mark(k);
    }
    launch_clear_dirty(d, L, s);
    mark(7);
    return PRGPU_OK;
}

int set_conf(prgpu_world* w, const prgpu_step_conf* conf) {
    if (!conf) return fail(w, PRGPU_EINVAL, "conf is NULL");
    if (conf->regPositionIters < 0 || conf->regPositionIters > kMaxPosIters || conf->regVelocityIters < 0)
        return fail(w, PRGPU_EINVAL, "iteration counts out of range (position iterations <= %d)", kMaxPosIters);
    if (conf->toiPositionIters < 0 || conf->toiVelocityIters < 0 || conf->maxToiRootIters < 0 ||
        conf->maxToiIters < 0 || conf->maxDistanceIters < 0 || conf->maxSubSteps < 0 || conf->maxSubSteps > 255)
        return fail(w, PRGPU_EINVAL, "time-of-impact iteration counts out of range (maxSubSteps <= 255)");
    if (!w->conf_valid || std::memcmp(&w->conf, conf, sizeof(*conf)) != 0) {
        static_assert(sizeof(prgpu_step_conf) == sizeof(DConf), "conf layout");
        CU(cudaMemcpyAsync(w->d_conf, conf, sizeof(DConf), cudaMemcpyHostToDevice, w->stream));
        w->conf = *conf;
        w->conf_valid = true;
    }
    return PRGPU_OK;
}

int check_device_error(prgpu_world* w) {
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (w->h_cnt->err) {
        const uint32_t code = w->h_cnt->err;
        return fail(w, (int)code, "device error %u at site %u", code, w->h_cnt->err_where);
    }
    return PRGPU_OK;
}

// Captures the launches `fn` enqueues on the world's stream into *g once.
template <class F>
int capture_once(prgpu_world* w, cudaGraphExec_t* g, F fn) {
    if (*g) return PRGPU_OK;
    CU(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
    fn();
    cudaGraph_t def = nullptr;
    const cudaError_t e1 = cudaStreamEndCapture(w->stream, &def);
    if (e1 != cudaSuccess) return fail(w, PRGPU_ECUDA, "graph capture: %s", cudaGetErrorString(e1));
    const cudaError_t e2 = cudaGraphInstantiate(g, def, 0);
    cudaGraphDestroy(def);
    if (e2 != cudaSuccess) return fail(w, PRGPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e2));
    return PRGPU_OK;
}

// Guard on the number of time-of-impact rounds of one step: every event adds a
// sub-step to one contact and contacts have at most maxSubSteps, so the loop
// ends long before this.
constexpr uint32_t kMaxToiRounds = 1u << 17;

// The time-of-impact phase of one step (AabbTreeWorld.cpp:1752-1831): round
// after round of one event per world until no world has an event left.  The
// host reads the device counters after each round to decide whether to go on.
int run_toi_phase(prgpu_world* w) {
    const DW& d = w->d;
    const Launch& L = w->L;
    cudaStream_t s = w->stream;
    int rc;
    if ((rc = capture_once(w, &w->toi_graph[0], [&] { launch_toi_begin(d, L, s); }))) return rc;
    if ((rc = capture_once(w, &w->toi_graph[1], [&] { launch_toi_round(d, L, s); }))) return rc;
    if ((rc = capture_once(w, &w->toi_graph[2], [&] { launch_toi_end(d, L, s); }))) return rc;
    CU(cudaGraphLaunch(w->toi_graph[0], s));
    for (uint32_t r = 0;; ++r) {
        CU(cudaGraphLaunch(w->toi_graph[1], s));
        CU(cudaMemcpyAsync(w->h_cnt, d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        if (w->h_cnt->err)
            return fail(w, (int)w->h_cnt->err, "device error %u at site %u", w->h_cnt->err, w->h_cnt->err_where);
        if (w->h_cnt->toi_events == 0u) break;
        if (r >= kMaxToiRounds) return fail(w, PRGPU_ETIMEOUT, "time-of-impact loop did not finish");
    }
    CU(cudaGraphLaunch(w->toi_graph[2], s));
    return PRGPU_OK;
}

// Launches the captured regular-phase step graph n times (capturing it first).
int launch_step_graphs(prgpu_world* w, int n) {
    if (!w->graph) {
        for (int k = 0; k < 8; ++k)
            if (!w->graph_ev[k]) CU(cudaEventCreate(&w->graph_ev[k]));
        CU(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(w, true, w->graph_ev, true);
        // the step's error word, for prgpu_step_async to read without waiting
        cudaMemcpyAsync(w->h_err, &w->d.cnt->err, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e1 = cudaStreamEndCapture(w->stream, &g);
        if (e1 != cudaSuccess) return fail(w, PRGPU_ECUDA, "graph capture: %s", cudaGetErrorString(e1));
        const cudaError_t e2 = cudaGraphInstantiate(&w->graph, g, 0);
        if (e2 != cudaSuccess) return fail(w, PRGPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e2));
        w->graph_def = g;
    }
    for (int i = 0; i < n; ++i) CU(cudaGraphLaunch(w->graph, w->stream));
    return PRGPU_OK;
}

// Moves a batch onto arrays of contact capacity C2 and candidate capacity K2:
// every array that is not per-step scratch is copied by position into its
// larger counterpart (alloc_world's order), so slots, keys and lists keep their
// indices and the batch continues exactly as it would have with the larger
// capacities from the start.
int grow_world(prgpu_world* w, uint32_t C2, uint32_t K2) {
    if (w->adj) return fail(w, PRGPU_ESTATE, "capacities cannot grow inside an adjoint window");
    int rc = drop_graph(w);
    if (rc) return rc;
    prgpu_world* n = new prgpu_world();
    n->device = w->device;
    n->d = w->d;
    n->d.contact_cap = C2;
    n->d.cand_cap = K2;
    WorldDims z = w->dims;
    z.C = C2;
    z.K = K2;
    rc = alloc_world(n, z);
    if (rc == PRGPU_OK && n->allocs.size() != w->allocs.size()) rc = PRGPU_ESTATE;
    for (size_t i = 0; rc == PRGPU_OK && i < w->allocs.size(); ++i) {
        if (w->alloc_scratch[i]) continue;
        const size_t b = std::min(w->alloc_bytes[i], n->alloc_bytes[i]);
        if (cudaMemcpyAsync(n->allocs[i], w->allocs[i], b, cudaMemcpyDeviceToDevice, w->stream) != cudaSuccess)
            rc = PRGPU_ECUDA;
    }
    float4* post_imp = nullptr;
    uint2* post_tag = nullptr;
    if (rc == PRGPU_OK && w->post_imp) {
        const size_t c0 = w->dims.C;
        if (cudaMalloc(&post_imp, sizeof(float4) * C2) != cudaSuccess ||
            cudaMalloc(&post_tag, sizeof(uint2) * C2) != cudaSuccess ||
            cudaMemsetAsync(post_tag, 0, sizeof(uint2) * C2, w->stream) != cudaSuccess ||
            cudaMemcpyAsync(post_imp, w->post_imp, sizeof(float4) * c0, cudaMemcpyDeviceToDevice, w->stream) != cudaSuccess ||
            cudaMemcpyAsync(post_tag, w->post_tag, sizeof(uint2) * c0, cudaMemcpyDeviceToDevice, w->stream) != cudaSuccess)
            rc = PRGPU_ECUDA;
    }
    if (rc == PRGPU_OK && cudaStreamSynchronize(w->stream) != cudaSuccess) rc = PRGPU_ECUDA;
    if (rc != PRGPU_OK) {
        if (post_imp) cudaFree(post_imp);
        if (post_tag) cudaFree(post_tag);
        prgpu_world_destroy(n);
        return fail(w, rc, "capacity growth to %u contacts failed", C2);
    }
    const bool records = w->d.cs_post_tag != nullptr;
    std::swap(w->allocs, n->allocs);
    std::swap(w->alloc_bytes, n->alloc_bytes);
    std::swap(w->alloc_scratch, n->alloc_scratch);
    std::swap(w->d_conf, n->d_conf);
    std::swap(w->d_stage, n->d_stage);
    w->d = n->d;
    w->dims = z;
    if (w->post_imp) {
        std::swap(w->post_imp, post_imp);
        std::swap(w->post_tag, post_tag);
        cudaFree(post_imp);
        cudaFree(post_tag);
    }
    w->d.cs_post = records ? w->post_imp : nullptr;
    w->d.cs_post_tag = records ? w->post_tag : nullptr;
    if (w->backup) { cudaFree(w->backup); w->backup = nullptr; w->backup_bytes = 0; }
    prgpu_world_destroy(n);  // the arrays the batch left
    return PRGPU_OK;
}

int run_steps(prgpu_world* w, const prgpu_step_conf* conf, int n, bool sync);

// Keeps the state before the step in w->backup (growth on).
int take_backup(prgpu_world* w) {
    const size_t bytes = snap_size(w);
    if (!w->backup || w->backup_bytes != bytes) {
        if (w->backup) cudaFree(w->backup);
        w->backup = nullptr;
        CU(cudaMalloc(&w->backup, bytes));
        w->backup_bytes = bytes;
    }
    return snap_copy(w, w->backup, true);
}

// Steps one by one; a step that runs out of contact or candidate capacity
// (PRGPU_ECAPACITY) is undone from the state kept before it, both capacities
// double, and the step runs again.
int run_steps_growing(prgpu_world* w, const prgpu_step_conf* conf, int n) {
    constexpr int kMaxDoublings = 16;
    for (int i = 0; i < n; ++i) {
        int rc = take_backup(w);
        if (rc) return rc;
        for (int attempt = 0;; ++attempt) {
            rc = run_steps(w, conf, 1, true);
            if (rc != PRGPU_ECAPACITY || attempt == kMaxDoublings) break;
            if ((rc = snap_copy(w, w->backup, false)) != PRGPU_OK) return rc;
            CU(cudaStreamSynchronize(w->stream));
            const uint32_t C2 = (uint32_t)std::min<uint64_t>(2ull * w->dims.C, 0x7fffffffull);
            const uint32_t K2 = (uint32_t)std::min<uint64_t>(2ull * w->dims.K, 0x7fffffffull);
            if ((rc = grow_world(w, C2, K2)) != PRGPU_OK) return rc;
            if ((rc = take_backup(w)) != PRGPU_OK) return rc;
        }
        if (rc) return rc;
    }
    return PRGPU_OK;
}

int run_steps(prgpu_world* w, const prgpu_step_conf* conf, int n, bool sync) {
    int rc = set_conf(w, conf);
    if (rc) return rc;
    if (n > 0) w->stepped = true;
    if (conf->deltaTime == 0.f) {
        for (int i = 0; i < n; ++i) enqueue_step(w, false);
        CU(cudaGetLastError());
    } else if (conf->doToi) {
        // the TOI loop reads the device counters between rounds: step by step
        for (int i = 0; i < n; ++i) {
            if ((rc = launch_step_graphs(w, 1)) != PRGPU_OK) return rc;
            if ((rc = run_toi_phase(w)) != PRGPU_OK) return rc;
        }
    } else if ((rc = launch_step_graphs(w, n)) != PRGPU_OK) {
        return rc;
    }
    if (sync) return check_device_error(w);
    return PRGPU_OK;
}

__global__ void k_apply_states(DW d, uint32_t first, uint32_t count, const float* pos3, const float* vel3) {
    GRID_LOOP(i, count) {
        const uint32_t b = first + i;
        uint32_t f = d.b_flags[b];
        if (pos3) {
            const float4 p = d.b_pos1[b];
            const float x = pos3[3 * i], y = pos3[3 * i + 1], a = pos3[3 * i + 2];
            if (x != p.x || y != p.y || a != p.z) {
                const float4 np = make_float4(x, y, a, 0.f);
                d.b_pos1[b] = np;
                d.b_pos0[b] = np;
                const float4 m = d.b_mass[b];
                const Xf xf = get_xf(x, y, a, mk(m.z, m.w));
                d.b_xf[b] = make_float4(xf.p.x, xf.p.y, xf.q.x, xf.q.y);
                f |= BF_DIRTY;
                d.cnt->dirty_any = 1u;
            }
        }
        if (vel3 && is_speedable(f)) {
            const float4 v = d.b_vel[b];
            const float vx = vel3[3 * i], vy = vel3[3 * i + 1], vw = vel3[3 * i + 2];
            if (vx != v.x || vy != v.y || vw != v.z) {
                d.b_vel[b] = make_float4(vx, vy, vw, 0.f);
                // Body::SetVelocity (Body.cpp:182-193): a non-zero velocity wakes the body
                if (vx != 0.f || vy != 0.f || vw != 0.f) { f |= BF_AWAKE; d.b_uat[b] = 0.f; }
            }
        }
        d.b_flags[b] = f;
    }
}

__global__ void k_gather_bodies(DW d, float* pos3, float* vel3, float* xf4, float* mass4, float* uat, uint32_t* flags) {
    GRID_LOOP(b, d.n_bodies) {
        const float4 p = d.b_pos1[b], v = d.b_vel[b], x = d.b_xf[b], m = d.b_mass[b];
        if (pos3) { pos3[3 * b] = p.x; pos3[3 * b + 1] = p.y; pos3[3 * b + 2] = p.z; }
        if (vel3) { vel3[3 * b] = v.x; vel3[3 * b + 1] = v.y; vel3[3 * b + 2] = v.z; }
        if (xf4) reinterpret_cast<float4*>(xf4)[b] = x;
        if (mass4) reinterpret_cast<float4*>(mass4)[b] = m;
        if (uat) uat[b] = d.b_uat[b];
        if (flags) flags[b] = (d.b_flags[b] & BF_AWAKE) ? 1u : 0u;
    }
}

__global__ void k_gather_contacts(DW d, uint32_t n, uint32_t* proxies2, uint32_t* bodies2, uint32_t* flags,
                                  int32_t* meta2, float* head4, float* pts8, uint32_t* feat2) {
    GRID_LOOP(i, n) {
        const uint32_t slot = d.c_slot[i];
        const uint2 pr = d.cs_proxy[slot], bd = d.cs_body[slot];
        if (proxies2) { proxies2[2 * i] = pr.x; proxies2[2 * i + 1] = pr.y; }
        if (bodies2) { bodies2[2 * i] = bd.x; bodies2[2 * i + 1] = bd.y; }
        if (flags) flags[i] = ((d.cs_flags[slot] & CF_TOUCHING) ? 1u : 0u) | ((d.cs_flags[slot] & CF_SENSOR) ? 2u : 0u);
        if (meta2) { const uint32_t m = d.m_meta[slot]; meta2[2 * i] = (int32_t)(m & 0xfu); meta2[2 * i + 1] = (int32_t)((m >> 4) & 0xfu); }
        if (head4) reinterpret_cast<float4*>(head4)[i] = d.m_head[slot];
        if (pts8) { reinterpret_cast<float4*>(pts8)[2 * i] = d.m_p0[slot]; reinterpret_cast<float4*>(pts8)[2 * i + 1] = d.m_p1[slot]; }
        if (feat2) { const uint2 c = d.m_cf[slot]; feat2[2 * i] = c.x; feat2[2 * i + 1] = c.y; }
    }
}

__global__ void k_gather_seq(DW d, uint32_t n, uint64_t* seq) {
    GRID_LOOP(i, n) seq[i] = d.cs_seq[d.c_slot[i]];
}

// Slot and the caller-settable fields of every live contact, in key order.
__global__ void k_gather_contact_state(DW d, uint32_t n, uint32_t* slots, float4* mat4) {
    GRID_LOOP(i, n) {
        const uint32_t slot = d.c_slot[i];
        slots[i] = slot;
        const float2 m = d.cs_mat[slot];
        mat4[i] = make_float4(m.x, m.y, d.cs_tspeed[slot], (d.cs_flags[slot] & CF_DISABLED) ? 0.f : 1.f);
    }
}

// The live contacts that the last step updated or solved: slot, then the
// phases that updated it (kUpd* bits), bit 3 if it was solved with its point
// count at bits 4-7 and the iteration argument at bits 8-15, and the solved
// impulses.  n_rec counts the records; nothing is written past cap.
__global__ void k_gather_solve_records(DW d, uint32_t n, uint32_t cap, uint32_t* n_rec, uint32_t* slots,
                                       uint32_t* info, float4* imp) {
    const uint32_t step = d.cnt->step_no;
    GRID_LOOP(i, n) {
        const uint32_t slot = d.c_slot[i];
        const uint32_t upd = d.cs_upd[slot];
        const uint32_t phases = ((upd >> 3) == step) ? (upd & 7u) : 0u;
        const uint2 tag = d.cs_post_tag ? d.cs_post_tag[slot] : make_uint2(0u, 0u);
        const bool posted = d.cs_post_tag && tag.x == step;
        if (!phases && !posted) continue;
        const uint32_t k = atomicAdd(n_rec, 1u);
        if (k >= cap) continue;
        slots[k] = slot;
        info[k] = phases | (posted ? 8u | ((tag.y & 0xffu) << 4) | (((tag.y >> 8) & 0xffu) << 8) : 0u);
        imp[k] = posted ? d.cs_post[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// SetContact / SetManifold on one slot; status 0 ok, 1 not a live contact,
// 2 the manifold's type or point count differs.
__global__ void k_set_contact(DW d, uint32_t slot, int enabled, float friction, float restitution, float tspeed,
                              uint32_t* status) {
    const uint32_t f = d.cs_flags[slot];
    if (!(f & CF_LIVE)) { *status = 1u; return; }
    d.cs_flags[slot] = enabled ? (f & ~CF_DISABLED) : (f | CF_DISABLED);
    d.cs_mat[slot] = make_float2(friction, restitution);
    d.cs_tspeed[slot] = tspeed;
    *status = 0u;
}
__global__ void k_set_manifold(DW d, uint32_t slot, int type, int count, float4 head, float4 p0, float4 p1,
                               uint32_t* status) {
    if (!(d.cs_flags[slot] & CF_LIVE)) { *status = 1u; return; }
    const uint32_t meta = d.m_meta[slot];
    if ((int)(meta & 0xfu) != type || (int)((meta >> 4) & 0xfu) != count) { *status = 2u; return; }
    d.m_head[slot] = head;
    d.m_p0[slot] = p0;
    d.m_p1[slot] = p1;
    *status = 0u;
}

}  // namespace

extern "C" {

int prgpu_abi_version(void) { return PRGPU_ABI_VERSION; }

int prgpu_default_step_conf(prgpu_step_conf* c) {
    if (!c) return PRGPU_EINVAL;
    // StepConf defaults (StepConf.hpp:59-161, Settings.hpp) in float arithmetic.
    const float Pi = 3.14159265358979323846264338327950288f;
    const float linearSlop = 0.005f;
    std::memset(c, 0, sizeof(*c));
    c->deltaTime = 1.0f / 60.0f;
    c->dtRatio = 1.0f;
    c->minStillTimeToSleep = 1.0f / 2.0f;
    c->linearSlop = linearSlop;
    c->angularSlop = (Pi * 2.0f) / 180.0f;
    c->regResolutionRate = 2.0f / 10.0f;
    c->regMinSeparation = -linearSlop * 3.0f;
    c->regMinMomentum = 0.0f / 100.0f;
    c->velocityThreshold = 1.0f;
    c->maxTranslation = 2.0f;
    c->maxRotation = 179.0f * ((1.0f * Pi) / 180.0f);
    c->maxLinearCorrection = 0.2f;
    c->maxAngularCorrection = (8.0f / 180.0f) * Pi;
    c->linearSleepTolerance = 0.01f;
    c->angularSleepTolerance = (Pi * 2.0f) / 180.0f;
    c->displaceMultiplier = 2.0f;
    c->aabbExtension = linearSlop * 20.0f;
    c->maxCirclesRatio = 10.0f;
    c->regVelocityIters = 8;
    c->regPositionIters = 3;
    c->doWarmStart = 1;
    c->doBlocksolve = 1;
    c->toiResolutionRate = 75.0f / 100.0f;
    c->toiMinSeparation = -linearSlop * 1.5f;
    c->toiMinMomentum = 0.0f / 100.0f;
    c->targetDepth = linearSlop * 3.0f;
    c->tolerance = linearSlop / 4.0f;
    c->toiVelocityIters = 8;
    c->toiPositionIters = 20;
    c->maxToiRootIters = 30;
    c->maxToiIters = 20;
    c->maxDistanceIters = 20;
    c->maxSubSteps = 8;
    c->doToi = 1;
    return PRGPU_OK;
}

int prgpu_convex_hull(const float* xy, int n, float linear_slop, float* out_xy) {
    if (!xy || !out_xy || n < 0) return -1;
    const float min_sep2 = linear_slop * linear_slop;
    std::vector<HV> pts;
    for (int i = 0; i < n; ++i) {
        const HV p = hv(xy[2 * i], xy[2 * i + 1]);
        bool dup = false;
        for (const HV& q : pts) {
            if (hmag2(p - q) <= min_sep2) { dup = true; break; }
        }
        if (!dup) pts.push_back(p);
    }
    const int m = (int)pts.size();
    if (m == 0) return 0;
    int i0 = 0;
    float max_x = pts[0].x;
    for (int i = 1; i < m; ++i) {
        const float x = pts[i].x;
        if ((max_x < x) || ((max_x == x) && (pts[i].y < pts[i0].y))) { max_x = x; i0 = i; }
    }
    std::vector<int> hull;
    int ih = i0;
    for (int guard = 0; guard <= m; ++guard) {
        hull.push_back(ih);
        int ie = 0;
        for (int j = 1; j < m; ++j) {
            if (ie == ih) { ie = j; continue; }
            const HV r = pts[ie] - pts[ih];
            const HV v = pts[j] - pts[ih];
            const float c = hcross(r, v);
            if ((c < 0.f) || ((c == 0.f) && (hmag2(v) > hmag2(r)))) ie = j;
        }
        ih = ie;
        if (ie == i0) break;
    }
    for (size_t k = 0; k < hull.size(); ++k) { out_xy[2 * k] = pts[hull[k]].x; out_xy[2 * k + 1] = pts[hull[k]].y; }
    return (int)hull.size();
}

int prgpu_time_of_impact(int device, uint32_t n, const uint32_t* nverts, const float* verts, const float* radius,
                         const float* sweeps, const prgpu_step_conf* conf, float* time_out, int32_t* iout4) {
    if (n == 0) return PRGPU_OK;
    if (!nverts || !verts || !radius || !sweeps || !conf || !time_out || !iout4) return PRGPU_EINVAL;
    std::vector<uint32_t> meta(2 * (size_t)n);
    std::vector<float4> vtx;
    std::vector<float> sw(2 * (size_t)n * 10);
    for (size_t k = 0; k < 2 * (size_t)n; ++k) {
        const uint32_t nv = nverts[k];
        if (nv < 1 || nv > 16u) return PRGPU_EINVAL;  // the shapes the step supports
        if (vtx.size() + nv >= (1u << 24)) return PRGPU_ECAPACITY;
        meta[k] = ((uint32_t)vtx.size() << 8) | nv;
        for (uint32_t i = 0; i < nv; ++i) {
            const size_t v = vtx.size();
            vtx.push_back(make_float4(verts[2 * v], verts[2 * v + 1], 0.f, 0.f));
        }
        for (int q = 0; q < 9; ++q) sw[k * 10 + q] = sweeps[k * 9 + q];
        sw[k * 10 + 9] = radius[k];
    }
    if (cudaSetDevice(device) != cudaSuccess) return PRGPU_ECUDA;
    float4* d_vtx = nullptr;
    uint32_t* d_meta = nullptr;
    float *d_sw = nullptr, *d_time = nullptr;
    int32_t* d_io = nullptr;
    DConf dc;
    static_assert(sizeof(prgpu_step_conf) == sizeof(DConf), "conf layout");
    std::memcpy(&dc, conf, sizeof(dc));
    cudaError_t e = cudaMalloc(&d_vtx, sizeof(float4) * vtx.size());
    if (e == cudaSuccess) e = cudaMalloc(&d_meta, sizeof(uint32_t) * meta.size());
    if (e == cudaSuccess) e = cudaMalloc(&d_sw, sizeof(float) * sw.size());
    if (e == cudaSuccess) e = cudaMalloc(&d_time, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&d_io, sizeof(int32_t) * 4 * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(d_vtx, vtx.data(), sizeof(float4) * vtx.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_meta, meta.data(), sizeof(uint32_t) * meta.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_sw, sw.data(), sizeof(float) * sw.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_toi_pairs(n, d_vtx, d_meta, d_sw, dc, d_time, d_io, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(time_out, d_time, sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(iout4, d_io, sizeof(int32_t) * 4 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d_vtx); cudaFree(d_meta); cudaFree(d_sw); cudaFree(d_time); cudaFree(d_io);
    return e == cudaSuccess ? PRGPU_OK : PRGPU_ECUDA;
}

int prgpu_prepare_bodies(const prgpu_batch_desc* ds, float* pos3, float* vel3, float* mass4) {
    if (!ds) return PRGPU_EINVAL;
    HostPrep hp;
    const int rc = prepare_host(ds, hp);
    if (rc) return rc;
    for (uint32_t b = 0; b < hp.N; ++b) {
        if (pos3) { pos3[3 * b] = hp.pos1[b].x; pos3[3 * b + 1] = hp.pos1[b].y; pos3[3 * b + 2] = hp.pos1[b].z; }
        if (vel3) { vel3[3 * b] = hp.vel[b].x; vel3[3 * b + 1] = hp.vel[b].y; vel3[3 * b + 2] = hp.vel[b].z; }
        if (mass4) { mass4[4 * b] = hp.mass[b].x; mass4[4 * b + 1] = hp.mass[b].y; mass4[4 * b + 2] = hp.mass[b].z; mass4[4 * b + 3] = hp.mass[b].w; }
    }
    return PRGPU_OK;
}

// Allocates every device array of a batch (in one fixed order: capacity growth
// copies a world's arrays onto a larger set by position in that order) and
// points w->d at them.
static int alloc_world(prgpu_world* w, const WorldDims& z) {
    DW& d = w->d;
    const uint32_t W = z.W, N = z.N, S = z.S, J = z.J, C = z.C, K = z.K;
    const uint32_t items = std::max<uint32_t>(std::max<uint32_t>(C + J, N + 1), S) + 1;
    int rc = 0;
#define AL(ptr, n) do { rc = dalloc(w, &(ptr), (size_t)(n)); if (rc) return rc; } while (0)
    // per-step scratch: every step writes it before reading it
#define ALS(ptr, n) do { rc = dalloc(w, &(ptr), (size_t)(n), true); if (rc) return rc; } while (0)
    AL(d.partial, 1024); AL(d.hist, 256 * 1025);  // digit rows of up to 1024 sort blocks, then the digit totals
    Counters* cnt;
    AL(cnt, 1);
    d.cnt = cnt;
    AL(w->d_conf, 1);
    d.conf = w->d_conf;
    AL(w->d_stage, (size_t)N * 8 + 16);
    uint32_t *w_body_off, *w_shape_off;
    AL(w_body_off, W + 1); AL(w_shape_off, W + 1);
    d.w_body_off = w_body_off; d.w_shape_off = w_shape_off;
    AL(d.w_root, W); AL(d.w_bounds, W);
    uint32_t* w_order;
    AL(w_order, W); d.w_order = w_order;
    // the TOI phase's state persists between steps when sub-stepping stops a phase
    AL(d.w_kc, W + 1); AL(d.w_kj, W + 1); ALS(d.w_toi, W); AL(d.w_toi_ep, W); AL(d.w_incomplete, W);
    AL(d.b_pos1, N); AL(d.b_pos0, N); AL(d.b_vel, N); AL(d.b_xf, N); AL(d.b_mass, N); AL(d.b_acc, N);
    AL(d.b_damp, N); AL(d.b_flags, N); AL(d.b_uat, N); AL(d.b_world, N); AL(d.b_island, N);
    // the TOI phase's own state: reset when the phase starts
    AL(d.b_alpha0, N); AL(d.b_toi_ep, N); AL(d.b_toi_rst, N);
    uint32_t *b_shape_off, *b_shapes;
    AL(b_shape_off, N + 1); AL(b_shapes, S);
    d.b_shape_off = b_shape_off; d.b_shapes = b_shapes;
    AL(d.b_jnt_off, N + 1); AL(d.b_jnt_other, z.JO); AL(d.b_jnt_cc, z.JC);
    AL(d.isl_awake, N); ALS(d.isl_sep, (size_t)N * kMaxPosIters); ALS(d.isl_jok, (size_t)N * kMaxPosIters); AL(d.isl_uat, N);
    AL(d.s_body, S); AL(d.s_meta, S); AL(d.s_voff, S); AL(d.s_radius, S); AL(d.s_rec, S); AL(d.s_mat, S);
    AL(d.s_filter, S);
    AL(d.s_group, S); AL(d.verts, z.V); AL(d.p_aabb, S); AL(d.p_moved, S); AL(d.moved_list, S);
    AL(d.j_bodies, 2 * J); AL(d.j_anchor, J); AL(d.j_param, J); AL(d.j_maxtorque, J); AL(d.j_flags, J);
    float4* j_extra_d;
    AL(j_extra_d, 2 * (size_t)J);
    d.j_extra = j_extra_d;
    float4* j_gear_d;
    AL(j_gear_d, 5 * (size_t)J);
    d.j_gear = j_gear_d;
    AL(d.j_r, J); AL(d.j_m0, J); AL(d.j_m1, J); AL(d.j_m2, J); AL(d.j_imp, J);
    AL(d.c_key, C); AL(d.c_slot, C); ALS(d.c_key_alt, C); ALS(d.c_slot_alt, C); AL(d.free_stack, C);
    AL(d.cs_proxy, C); AL(d.cs_body, C); AL(d.cs_flags, C); AL(d.cs_mat, C); AL(d.cs_tspeed, C);
    AL(d.cs_colour, C); AL(d.j_colour, J); AL(d.cs_toi, C); AL(d.cs_seq, C); AL(d.cs_prio, C); AL(d.cs_upd, C);
    AL(d.cs_toi_ep, C); AL(d.cs_toi_at, C); ALS(d.t_key, C); ALS(d.t_slot, C);
    AL(d.m_head, C); AL(d.m_p0, C); AL(d.m_p1, C); AL(d.m_meta, C); AL(d.m_cf, C);
    ALS(d.n_key, K); ALS(d.n_key_alt, K); ALS(d.n_val, K); ALS(d.n_val_alt, K);
    AL(d.l_key, S); AL(d.l_key_alt, S); AL(d.l_idx, S); AL(d.l_idx_alt, S); AL(d.l_leaf_box, S);
    AL(d.l_node_box, S); AL(d.l_left, S); AL(d.l_right, S); AL(d.l_parent, 2 * (size_t)S); AL(d.l_range, 2 * (size_t)S);
    AL(d.l_visit, S); AL(d.l_inv, S); ALS(d.c_first, (size_t)S + 1);
    ALS(d.k_list, C + J); ALS(d.k_colour, C + J); ALS(d.k_tent, C + J); ALS(d.k_order, C + J);
    ALS(d.t_id, C + J);
    ALS(d.k_prio, C + J);
    AL(d.inc_off, N + 1); AL(d.inc_cur, N + 1); ALS(d.inc_list, 2 * (size_t)C + 4 * (size_t)J);
    ALS(d.vc0, C + J); ALS(d.vc1, C + J); ALS(d.pc, C + J);
    ALS(d.flags, items); ALS(d.scan, items);
#undef AL
#undef ALS
    return PRGPU_OK;
}

int prgpu_world_create(const prgpu_batch_desc* ds, int device, prgpu_world** out) {
    if (!ds || !out) return PRGPU_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return PRGPU_ENOTREADY;
    prgpu_world* w = new prgpu_world();
    w->device = device;
    auto bail = [&](int rc) { prgpu_world_destroy(w); return rc; };
    if (cudaSetDevice(device) != cudaSuccess) return bail(PRGPU_ECUDA);
    HostPrep hp;
    {
        const int prc = prepare_host(ds, hp);
        if (prc) return bail(fail(w, prc, "invalid batch description"));
    }
    const uint32_t W = hp.W, N = hp.N, S = hp.S, J = hp.J;
    auto& body_off = hp.body_off; auto& shape_off = hp.shape_off; auto& body_world = hp.body_world;
    auto& pos1 = hp.pos1; auto& vel = hp.vel; auto& mass = hp.mass; auto& acc = hp.acc; auto& damp = hp.damp;
    auto& bflags = hp.bflags; auto& s_meta = hp.s_meta; auto& s_voff = hp.s_voff; auto& s_filter = hp.s_filter;
    auto& s_body = hp.s_body; auto& p_state = hp.p_state; auto& s_group = hp.s_group; auto& s_radius = hp.s_radius;
    auto& s_mat = hp.s_mat; auto& vtx = hp.vtx; auto& joff = hp.joff; auto& jother = hp.jother; auto& jcc = hp.jcc;
    auto& j_anchor = hp.j_anchor; auto& j_param = hp.j_param; auto& j_zero = hp.j_zero; auto& j_maxtorque = hp.j_maxtorque;
    auto& j_bodies = hp.j_bodies; auto& j_flags = hp.j_flags;
    // ---- capacities
    const uint64_t ccap = ds->contact_capacity ? ds->contact_capacity : (uint64_t)8 * S + 4096;
    const uint64_t kcap = ds->candidate_capacity ? ds->candidate_capacity : (uint64_t)8 * S + 4096;
    if (ccap > 0x7fffffffull || kcap > 0x7fffffffull) return bail(PRGPU_ECAPACITY);
    const uint32_t C = (uint32_t)ccap, K = (uint32_t)kcap;
    DW& d = w->d;
    d.n_worlds = W; d.n_bodies = N; d.n_shapes = S; d.n_joints = J; d.n_verts = (uint32_t)vtx.size();
    d.contact_cap = C; d.cand_cap = K;
    d.key_bits = (uint32_t)bits_for((uint64_t)S + 1);
    if (2 * d.key_bits > 64) return bail(PRGPU_ECAPACITY);
    d.world_bits = (uint32_t)bits_for((uint64_t)W + 1);
    if (30 + d.world_bits > 64) return bail(PRGPU_ECAPACITY);
    int rc = 0;
    {
        WorldDims z;
        z.W = W; z.N = N; z.S = S; z.J = J; z.C = C; z.K = K; z.V = (uint32_t)vtx.size();
        z.JO = (uint32_t)jother.size(); z.JC = (uint32_t)jcc.size();
        w->dims = z;
        if ((rc = alloc_world(w, z)) != PRGPU_OK) return bail(rc);
    }
    uint32_t* w_body_off = const_cast<uint32_t*>(d.w_body_off);
    uint32_t* w_shape_off = const_cast<uint32_t*>(d.w_shape_off);
    uint32_t* w_order = const_cast<uint32_t*>(d.w_order);
    uint32_t* b_shape_off = const_cast<uint32_t*>(d.b_shape_off);
    uint32_t* b_shapes = const_cast<uint32_t*>(d.b_shapes);
    float4* j_extra_d = const_cast<float4*>(d.j_extra);
    float4* j_gear_d = const_cast<float4*>(d.j_gear);
    w->L.prims.sm_count = 1;
    {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return bail(PRGPU_ECUDA);
        w->L.prims.sm_count = prop.multiProcessorCount;
    }
    w->L.prims.grid = std::min(1024, 2 * w->L.prims.sm_count);
    (void)radix_coop_grid(w->L.prims);  // occupancy query before any stream capture
    if (cudaMallocHost(&w->h_cnt, sizeof(Counters)) != cudaSuccess) return bail(PRGPU_ECUDA);
    if (cudaMallocHost(&w->h_err, 2 * sizeof(uint32_t)) != cudaSuccess) return bail(PRGPU_ECUDA);
    w->h_err[0] = w->h_err[1] = 0u;
    w->L.threads = 256;
    w->L.grid = w->L.prims.sm_count * 8;
    w->L.coop_threads = 256;
    const int per_sm = coop_blocks_per_sm(w->L.coop_threads);
    if (per_sm < 1) return bail(fail(w, PRGPU_ECUDA, "cooperative kernels cannot be resident"));
    w->L.coop_grid = w->L.prims.sm_count * std::min(per_sm, 4);
    {
        d.stage_bytes = kStageBytes;
        const int wps = world_blocks_per_sm(d.stage_bytes);
        if (wps < 1) return bail(fail(w, PRGPU_ECUDA, "per-world sweep kernel cannot be resident"));
        for (uint32_t sb : kStageChoices) world_blocks_per_sm(sb);  // raise the attribute once
        if (wps < 1) return bail(fail(w, PRGPU_ECUDA, "per-world sweep kernel cannot be resident"));
        w->L.world_grid = w->L.prims.sm_count * wps;
        w->L.per_world = W >= kPerWorldMinWorlds;
    }
    // worlds by decreasing body count, ties by index: the per-world sweeps
    // start the longest worlds first
    std::vector<uint32_t> order(W);
    for (uint32_t i = 0; i < W; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return body_off[a + 1] - body_off[a] > body_off[b + 1] - body_off[b];
    });
    w->order_nb.resize(W);
    for (uint32_t i = 0; i < W; ++i) w->order_nb[i] = body_off[order[i] + 1] - body_off[order[i]];
    w->L.isl_big_worlds = W > 0 && w->order_nb[0] > kIslSmemBodiesMax;
    w->warp_world_max = kWarpWorldMaxBodies;
    count_world_classes(w);
    if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(PRGPU_ECUDA);
    // ---- uploads
    auto up = [&](void* dst, const void* src, size_t bytes) -> bool {
        return bytes == 0 || cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, w->stream) == cudaSuccess;
    };
    bool ok = true;
    ok &= up(w_body_off, body_off.data(), sizeof(uint32_t) * (W + 1));
    ok &= up(w_shape_off, shape_off.data(), sizeof(uint32_t) * (W + 1));
    ok &= up(w_order, order.data(), sizeof(uint32_t) * W);
    ok &= up(d.b_pos1, pos1.data(), sizeof(float4) * N);
    ok &= up(d.b_vel, vel.data(), sizeof(float4) * N);
    ok &= up(d.b_mass, mass.data(), sizeof(float4) * N);
    ok &= up(d.b_acc, acc.data(), sizeof(float4) * N);
    ok &= up(d.b_damp, damp.data(), sizeof(float2) * N);
    ok &= up(d.b_flags, bflags.data(), sizeof(uint32_t) * N);
    ok &= up(d.b_world, body_world.data(), sizeof(uint32_t) * N);
    ok &= up(d.b_jnt_off, joff.data(), sizeof(uint32_t) * (N + 1));
    ok &= up(d.b_jnt_other, jother.data(), sizeof(uint32_t) * jother.size());
    ok &= up(d.b_jnt_cc, jcc.data(), sizeof(uint32_t) * jcc.size());
    ok &= up(d.s_body, s_body.data(), sizeof(uint32_t) * S);
    // body -> shapes, in shape order
    std::vector<uint32_t> bs_off(N + 1, 0u), bs_idx(S);
    for (uint32_t p = 0; p < S; ++p) ++bs_off[s_body[p] + 1];
    for (uint32_t b = 0; b < N; ++b) bs_off[b + 1] += bs_off[b];
    {
        std::vector<uint32_t> cur(bs_off.begin(), bs_off.end() - 1);
        for (uint32_t p = 0; p < S; ++p) bs_idx[cur[s_body[p]]++] = p;
    }
    ok &= up(b_shape_off, bs_off.data(), sizeof(uint32_t) * (N + 1));
    ok &= up(b_shapes, bs_idx.data(), sizeof(uint32_t) * S);
    ok &= up(d.s_meta, s_meta.data(), sizeof(uint32_t) * S);
    w->L.sensors = std::any_of(s_meta.begin(), s_meta.end(), [](uint32_t m) { return (m & kShapeSensor) != 0u; });
    ok &= up(d.s_voff, s_voff.data(), sizeof(uint32_t) * S);
    ok &= up(d.s_radius, s_radius.data(), sizeof(float) * S);
    {
        std::vector<uint4> rec(S);
        for (uint32_t p = 0; p < S; ++p) {
            uint32_t r;
            std::memcpy(&r, &s_radius[p], sizeof r);
            rec[p] = make_uint4(s_meta[p], s_voff[p], r, s_body[p]);
        }
        ok &= up(d.s_rec, rec.data(), sizeof(uint4) * S);
    }
    ok &= up(d.s_mat, s_mat.data(), sizeof(float2) * S);
    ok &= up(d.s_filter, s_filter.data(), sizeof(uint32_t) * S);
    ok &= up(d.s_group, s_group.data(), sizeof(int32_t) * S);
    ok &= up(d.verts, vtx.data(), sizeof(float4) * vtx.size());
    ok &= up(d.p_moved, p_state.data(), sizeof(uint32_t) * S);
    ok &= up(d.j_bodies, j_bodies.data(), sizeof(uint32_t) * 2 * J);
    ok &= up(d.j_anchor, j_anchor.data(), sizeof(float4) * J);
    ok &= up(d.j_param, j_param.data(), sizeof(float4) * J);
    ok &= up(j_extra_d, hp.j_extra.data(), sizeof(float4) * 2 * J);
    ok &= up(j_gear_d, hp.j_gear.data(), sizeof(float4) * 5 * J);
    ok &= up(d.j_maxtorque, j_maxtorque.data(), sizeof(float) * J);
    ok &= up(d.j_flags, j_flags.data(), sizeof(uint32_t) * J);
    ok &= up(d.j_imp, j_zero.data(), sizeof(float4) * J);
    ok &= up(d.j_m1, j_zero.data(), sizeof(float4) * J);
    ok &= up(d.j_m2, j_zero.data(), sizeof(float4) * J);
    ok &= cudaMemsetAsync(d.b_uat, 0, sizeof(float) * N, w->stream) == cudaSuccess;
    ok &= cudaMemsetAsync(d.b_alpha0, 0, sizeof(float) * N, w->stream) == cudaSuccess;
    ok &= cudaMemsetAsync(d.w_incomplete, 0, sizeof(uint32_t) * W, w->stream) == cudaSuccess;
    ok &= cudaMemsetAsync(d.cnt, 0, sizeof(Counters), w->stream) == cudaSuccess;
    ok &= cudaMemsetAsync(d.cs_upd, 0, sizeof(uint32_t) * std::max<uint32_t>(C, 1), w->stream) == cudaSuccess;
    ok &= cudaMemsetAsync(d.j_colour, 0xff, sizeof(uint32_t) * std::max<uint32_t>(J, 1), w->stream) == cudaSuccess;
    if (!ok) return bail(fail(w, PRGPU_ECUDA, "upload failed"));
    launch_init_bodies(d, w->L, w->stream);
    if (cudaStreamSynchronize(w->stream) != cudaSuccess) return bail(PRGPU_ECUDA);
    if (cudaGetLastError() != cudaSuccess) return bail(PRGPU_ECUDA);
    *out = w;
    return PRGPU_OK;
}

void adjoint_close(prgpu_world* w);

int prgpu_world_destroy(prgpu_world* w) {
    if (!w) return PRGPU_OK;
    cudaSetDevice(w->device);
    if (w->stream) cudaStreamSynchronize(w->stream);
    adjoint_close(w);
    if (w->graph) cudaGraphExecDestroy(w->graph);
    for (int k = 0; k < 8; ++k)
        if (w->graph_ev[k]) cudaEventDestroy(w->graph_ev[k]);
    if (w->graph_def) cudaGraphDestroy(w->graph_def);
    for (auto g : w->toi_graph)
        if (g) cudaGraphExecDestroy(g);
    for (void* p : w->allocs) cudaFree(p);
    if (w->post_imp) cudaFree(w->post_imp);
    if (w->post_tag) cudaFree(w->post_tag);
    if (w->backup) cudaFree(w->backup);
    if (w->h_cnt) cudaFreeHost(w->h_cnt);
    if (w->h_err) cudaFreeHost(w->h_err);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
    return PRGPU_OK;
}

void fill_stats(const Counters& c, prgpu_step_stats* st) {
    st->contactsAdded = c.st_contacts_added;
    st->contactsDestroyed = c.st_contacts_destroyed;
    st->contactsUpdated = c.st_contacts_updated;
    st->islandsFound = c.st_islands_found;
    st->islandsSolved = c.st_islands_solved;
    st->bodiesSlept = c.st_bodies_slept;
    st->proxiesMoved = c.st_proxies_moved;
    st->sumPosIters = c.st_sum_pos_iters;
    st->liveContacts = c.n_live;
    st->activeConstraints = c.n_active;
    st->colours = c.n_colours;
    st->serialConstraints = c.colour_off[kSerialColour + 1] - c.colour_off[kSerialColour];
    st->minSeparation = c.st_min_separation;
    st->maxIncImpulse = c.st_max_inc_impulse;
    st->toiIslandsFound = c.st_toi_islands_found;
    st->toiIslandsSolved = c.st_toi_islands_solved;
    st->toiContactsFound = c.st_toi_found;
    st->toiContactsAtMaxSubSteps = c.st_toi_at_max_substeps;
    st->toiContactsUpdatedToi = c.st_toi_updated_toi;
    st->toiContactsUpdatedTouching = c.st_toi_updated_touching;
    st->toiContactsSkippedTouching = c.st_toi_skipped_touching;
    st->toiContactsAdded = c.st_toi_contacts_added;
    st->toiProxiesMoved = c.st_toi_proxies_moved;
    st->toiSumPosIters = c.st_toi_sum_pos_iters;
    st->toiSumVelIters = c.st_toi_sum_vel_iters;
    st->toiMaxDistIters = c.st_toi_max_dist_iters;
    st->toiMaxToiIters = c.st_toi_max_toi_iters;
    st->toiMaxRootIters = c.st_toi_max_root_iters;
    st->toiRounds = c.toi_rounds;
    st->toiMinSeparation = c.st_toi_min_separation;
    st->toiMaxIncImpulse = c.st_toi_max_inc_impulse;
    st->bodiesSolved = c.st_bodies_solved;
}

int prgpu_step(prgpu_world* w, const prgpu_step_conf* conf, prgpu_step_stats* st) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    const int rc = w->grow ? run_steps_growing(w, conf, 1) : run_steps(w, conf, 1, true);
    if (rc) return rc;
    if (st) fill_stats(*w->h_cnt, st);
    return PRGPU_OK;
}

int prgpu_step_n(prgpu_world* w, const prgpu_step_conf* conf, int n) {
    if (!w || n < 0) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    return w->grow ? run_steps_growing(w, conf, n) : run_steps(w, conf, n, true);
}

int prgpu_set_capacity_growth(prgpu_world* w, int enabled) {
    if (!w) return PRGPU_EINVAL;
    w->grow = enabled != 0;
    if (!w->grow && w->backup) {
        CU(cudaSetDevice(w->device));
        cudaFree(w->backup);
        w->backup = nullptr;
        w->backup_bytes = 0;
    }
    return PRGPU_OK;
}

int prgpu_get_capacities(prgpu_world* w, uint32_t* contacts, uint32_t* candidates) {
    if (!w) return PRGPU_EINVAL;
    if (contacts) *contacts = w->d.contact_cap;
    if (candidates) *candidates = w->d.cand_cap;
    return PRGPU_OK;
}

int prgpu_set_sub_stepping(prgpu_world* w, int enabled) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    const uint32_t v = enabled ? 1u : 0u;
    CU(cudaMemcpyAsync(&w->d.cnt->sub_stepping, &v, sizeof(v), cudaMemcpyHostToDevice, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_get_step_complete(prgpu_world* w, uint32_t world, int* complete) {
    if (!w || !complete) return PRGPU_EINVAL;
    if (world >= w->d.n_worlds) return fail(w, PRGPU_EINVAL, "world %u out of range", world);
    CU(cudaSetDevice(w->device));
    uint32_t v = 0;
    CU(cudaMemcpyAsync(&v, w->d.w_incomplete + world, sizeof(v), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    *complete = v ? 0 : 1;
    return PRGPU_OK;
}

int prgpu_set_wait_limit(prgpu_world* w, uint32_t spins) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(&w->d.cnt->wait_limit, &spins, sizeof(spins), cudaMemcpyHostToDevice, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_step_profiled(prgpu_world* w, const prgpu_step_conf* conf, float* phase_ms, int n_phases,
                        prgpu_step_stats* st) {
    if (!w || !conf) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    int rc = set_conf(w, conf);
    if (rc) return rc;
    w->stepped = true;
    cudaEvent_t ev[kPhases + 1];
    for (int k = 0; k <= kPhases; ++k) CU(cudaEventCreate(&ev[k]));
    enqueue_step(w, conf->deltaTime != 0.f, ev);
    CU(cudaGetLastError());
    if (conf->deltaTime != 0.f && conf->doToi && (rc = run_toi_phase(w)) != PRGPU_OK) {
        for (int k = 0; k <= kPhases; ++k) cudaEventDestroy(ev[k]);
        return rc;
    }
    rc = check_device_error(w);
    if (!rc && phase_ms) {
        for (int k = 0; k < n_phases && k < kPhases; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            phase_ms[k] = ms;
        }
    }
    for (int k = 0; k <= kPhases; ++k) cudaEventDestroy(ev[k]);
    if (!rc && st) fill_stats(*w->h_cnt, st);
    return rc;
}

int prgpu_graph_kernel_count(prgpu_world* w, uint32_t* n_kernels) {
    if (!w || !n_kernels) return PRGPU_EINVAL;
    if (!w->graph_def) return fail(w, PRGPU_ESTATE, "no captured step yet");
    size_t n = 0;
    CU(cudaGraphGetNodes(w->graph_def, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    CU(cudaGraphGetNodes(w->graph_def, nodes.data(), &n));
    uint32_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType t;
        CU(cudaGraphNodeGetType(nodes[i], &t));
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    *n_kernels = k;
    return PRGPU_OK;
}

int prgpu_last_step_phase_ms(prgpu_world* w, float* phase_ms, int n_phases) {
    if (!w || !phase_ms) return PRGPU_EINVAL;
    if (!w->graph) return fail(w, PRGPU_ESTATE, "no captured step has run yet");
    CU(cudaSetDevice(w->device));
    CU(cudaStreamSynchronize(w->stream));
    for (int k = 0; k < n_phases && k < kPhases + 1; ++k) {
        float ms = 0.f;
        // phase k of the last replay; index kPhases gives the whole step
        const int a = (k < kPhases) ? k : 0, b = (k < kPhases) ? k + 1 : kPhases;
        CU(cudaEventElapsedTime(&ms, w->graph_ev[a], w->graph_ev[b]));
        phase_ms[k] = ms;
    }
    return PRGPU_OK;
}

int prgpu_set_sweep_mode(prgpu_world* w, int mode) {
    if (!w) return PRGPU_EINVAL;
    if (mode < PRGPU_SWEEPS_AUTO || mode > PRGPU_SWEEPS_PER_WORLD) return fail(w, PRGPU_EINVAL, "unknown sweep mode %d", mode);
    const bool per_world = (mode == PRGPU_SWEEPS_AUTO) ? (w->d.n_worlds >= kPerWorldMinWorlds)
                                                         : (mode == PRGPU_SWEEPS_PER_WORLD);
    if (per_world == w->L.per_world) return PRGPU_OK;
    const int rc = drop_graph(w);
    if (rc) return rc;
    w->L.per_world = per_world;
    return PRGPU_OK;
}

int prgpu_set_warp_world_max_bodies(prgpu_world* w, uint32_t max_bodies) {
    if (!w) return PRGPU_EINVAL;
    if (max_bodies == w->warp_world_max) return PRGPU_OK;
    const int rc = drop_graph(w);
    if (rc) return rc;
    w->warp_world_max = max_bodies;
    count_world_classes(w);
    return PRGPU_OK;
}

constexpr size_t kAutotuneRetime = 3;  // candidates the autotuner times a second time

int prgpu_autotune(prgpu_world* w, const prgpu_step_conf* conf, int steps_per_candidate, prgpu_schedule* best) {
    if (!w || !conf || steps_per_candidate < 1) return PRGPU_EINVAL;
    if (conf->deltaTime == 0.f) return fail(w, PRGPU_EINVAL, "autotune needs a step with deltaTime > 0");
    CU(cudaSetDevice(w->device));
    struct Cand { int mode; uint32_t warp_max; uint32_t stage; uint32_t group_max; };
    std::vector<Cand> cands = {{PRGPU_SWEEPS_GRID, w->warp_world_max, w->d.stage_bytes, 0u}};
    if (w->d.n_worlds > 1) {
        for (uint32_t sb : kStageChoices)
            for (uint32_t m : {0u, 64u, 128u, 256u, 1024u}) cands.push_back({PRGPU_SWEEPS_PER_WORLD, m, sb, 0u});
        // worlds up to 256, 512 or 1024 bodies swept by groups of 64 threads
        for (uint32_t m : {0u, 64u})
            for (uint32_t g : {256u, 512u, 1024u}) cands.push_back({PRGPU_SWEEPS_PER_WORLD, m, 0u, g});
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    // Times one candidate: a capturing step, then steps_per_candidate timed steps.
    auto time_cand = [&](const Cand& cd, float* ms) -> int {
        int r;
        if ((r = prgpu_set_sweep_mode(w, cd.mode)) != PRGPU_OK) return r;
        if ((r = prgpu_set_warp_world_max_bodies(w, cd.warp_max)) != PRGPU_OK) return r;
        if ((r = prgpu_set_group_world_max_bodies(w, cd.group_max)) != PRGPU_OK) return r;
        if ((r = prgpu_set_stage_bytes(w, cd.stage)) != PRGPU_OK) return r;
        if ((r = run_steps(w, conf, 1, true)) != PRGPU_OK) return r;  // captures the candidate's step
        if (cudaEventRecord(e0, w->stream) != cudaSuccess) return PRGPU_ECUDA;
        if ((r = run_steps(w, conf, steps_per_candidate, false)) != PRGPU_OK) return r;
        if (cudaEventRecord(e1, w->stream) != cudaSuccess) return PRGPU_ECUDA;
        if ((r = check_device_error(w)) != PRGPU_OK) return r;
        if (cudaEventElapsedTime(ms, e0, e1) != cudaSuccess) return PRGPU_ECUDA;
        *ms /= (float)steps_per_candidate;
        return PRGPU_OK;
    };
    // Every candidate once, then the kAutotuneRetime fastest once more (a few per
    // cent separate close candidates, about what two steps vary by); each keeps
    // its faster timing.
    std::vector<float> ms(cands.size(), 0.f);
    int rc = PRGPU_OK;
    for (size_t i = 0; i < cands.size() && rc == PRGPU_OK; ++i) rc = time_cand(cands[i], &ms[i]);
    if (rc == PRGPU_OK && cands.size() > 1) {
        std::vector<size_t> rank(cands.size());
        for (size_t i = 0; i < rank.size(); ++i) rank[i] = i;
        std::stable_sort(rank.begin(), rank.end(), [&](size_t a, size_t b) { return ms[a] < ms[b]; });
        for (size_t k = 0; k < std::min<size_t>(kAutotuneRetime, rank.size()) && rc == PRGPU_OK; ++k) {
            float again = 0.f;
            rc = time_cand(cands[rank[k]], &again);
            ms[rank[k]] = std::min(ms[rank[k]], again);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    size_t fastest = 0;
    for (size_t i = 1; i < cands.size(); ++i)
        if (ms[i] < ms[fastest]) fastest = i;
    const Cand pick = cands[fastest];
    const float best_ms = ms[fastest];
    if ((rc = prgpu_set_sweep_mode(w, pick.mode)) != PRGPU_OK) return rc;
    if ((rc = prgpu_set_warp_world_max_bodies(w, pick.warp_max)) != PRGPU_OK) return rc;
    if ((rc = prgpu_set_group_world_max_bodies(w, pick.group_max)) != PRGPU_OK) return rc;
    if ((rc = prgpu_set_stage_bytes(w, pick.stage)) != PRGPU_OK) return rc;
    if (best) {
        best->sweep_mode = pick.mode;
        best->warp_world_max_bodies = pick.warp_max;
        best->group_world_max_bodies = pick.group_max;
        best->stage_bytes = pick.stage;
        best->step_ms = best_ms;
    }
    return PRGPU_OK;
}

int prgpu_set_stage_bytes(prgpu_world* w, uint32_t bytes) {
    if (!w) return PRGPU_EINVAL;
    if (bytes % 128u != 0u || bytes > 200u * 1024u) return fail(w, PRGPU_EINVAL, "stage bytes must be a multiple of 128, <= 200 KiB");
    if (bytes == w->d.stage_bytes) return PRGPU_OK;
    CU(cudaSetDevice(w->device));
    const int wps = world_blocks_per_sm(bytes);
    if (wps < 1) return fail(w, PRGPU_EINVAL, "per-world solver cannot be resident with %u bytes of staging", bytes);
    const int rc = drop_graph(w);
    if (rc) return rc;
    w->d.stage_bytes = bytes;
    w->L.world_grid = w->L.prims.sm_count * wps;
    return PRGPU_OK;
}

int prgpu_get_stage_bytes(prgpu_world* w, uint32_t* bytes) {
    if (!w || !bytes) return PRGPU_EINVAL;
    *bytes = w->d.stage_bytes;
    return PRGPU_OK;
}

int prgpu_set_group_world_max_bodies(prgpu_world* w, uint32_t max_bodies) {
    if (!w) return PRGPU_EINVAL;
    if (max_bodies == w->group_world_max) return PRGPU_OK;
    const int rc = drop_graph(w);
    if (rc) return rc;
    w->group_world_max = max_bodies;
    count_world_classes(w);
    return PRGPU_OK;
}

int prgpu_get_group_world_max_bodies(prgpu_world* w, uint32_t* max_bodies) {
    if (!w || !max_bodies) return PRGPU_EINVAL;
    *max_bodies = w->group_world_max;
    return PRGPU_OK;
}

int prgpu_get_warp_world_max_bodies(prgpu_world* w, uint32_t* max_bodies) {
    if (!w || !max_bodies) return PRGPU_EINVAL;
    *max_bodies = w->warp_world_max;
    return PRGPU_OK;
}

int prgpu_get_sweep_mode(prgpu_world* w, int* mode) {
    if (!w || !mode) return PRGPU_EINVAL;
    *mode = w->L.per_world ? PRGPU_SWEEPS_PER_WORLD : PRGPU_SWEEPS_GRID;
    return PRGPU_OK;
}

int prgpu_step_async(prgpu_world* w, const prgpu_step_conf* conf, int n) {
    if (!w || n < 0) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    // an error of a step that has already finished (its graph copied the error
    // word to pinned memory as it ended) stops the caller before more are queued
    const volatile uint32_t* he = w->h_err;
    if (he[0]) return fail(w, (int)he[0], "device error %u at site %u (an earlier step)", he[0], he[1]);
    return run_steps(w, conf, n, false);
}

int prgpu_get_body_steps(prgpu_world* w, uint64_t* total) {
    if (!w || !total) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    *total = w->h_cnt->body_steps;
    return PRGPU_OK;
}

int prgpu_synchronize(prgpu_world* w) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    return check_device_error(w);
}

int prgpu_get_counts(prgpu_world* w, uint32_t* nw, uint32_t* nb, uint32_t* ns, uint32_t* nj, uint32_t* nc) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    if (nc) {
        CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        *nc = w->h_cnt->n_live;
    }
    if (nw) *nw = w->d.n_worlds;
    if (nb) *nb = w->d.n_bodies;
    if (ns) *ns = w->d.n_shapes;
    if (nj) *nj = w->d.n_joints;
    return PRGPU_OK;
}

int prgpu_download_bodies(prgpu_world* w, float* pos3, float* vel3, float* xf4, float* mass4, float* uat,
                          uint32_t* flags) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    const uint32_t N = w->d.n_bodies;
    float* base = w->d_stage;
    float* dpos = pos3 ? base : nullptr;
    float* dvel = vel3 ? base + (size_t)3 * N : nullptr;
    std::vector<float> tmp;
    k_gather_bodies<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, dpos, dvel, nullptr, nullptr, nullptr, nullptr);
    CU(cudaGetLastError());
    if (pos3) CU(cudaMemcpyAsync(pos3, dpos, sizeof(float) * 3 * N, cudaMemcpyDeviceToHost, w->stream));
    if (vel3) CU(cudaMemcpyAsync(vel3, dvel, sizeof(float) * 3 * N, cudaMemcpyDeviceToHost, w->stream));
    if (xf4) CU(cudaMemcpyAsync(xf4, w->d.b_xf, sizeof(float4) * N, cudaMemcpyDeviceToHost, w->stream));
    if (mass4) CU(cudaMemcpyAsync(mass4, w->d.b_mass, sizeof(float4) * N, cudaMemcpyDeviceToHost, w->stream));
    if (uat) CU(cudaMemcpyAsync(uat, w->d.b_uat, sizeof(float) * N, cudaMemcpyDeviceToHost, w->stream));
    if (flags) {
        std::vector<uint32_t> f(N);
        CU(cudaMemcpyAsync(f.data(), w->d.b_flags, sizeof(uint32_t) * N, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        for (uint32_t b = 0; b < N; ++b) flags[b] = (f[b] & BF_AWAKE) ? 1u : 0u;
    }
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_upload_body_states(prgpu_world* w, uint32_t first, uint32_t count, const float* pos3, const float* vel3) {
    if (!w) return PRGPU_EINVAL;
    if ((uint64_t)first + count > w->d.n_bodies) return fail(w, PRGPU_EINVAL, "body range out of bounds");
    CU(cudaSetDevice(w->device));
    float* dpos = pos3 ? w->d_stage : nullptr;
    float* dvel = vel3 ? w->d_stage + (size_t)3 * w->d.n_bodies : nullptr;
    if (pos3) CU(cudaMemcpyAsync(dpos, pos3, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, w->stream));
    if (vel3) CU(cudaMemcpyAsync(dvel, vel3, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, w->stream));
    k_apply_states<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, first, count, dpos, dvel);
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

// Device scratch from cudaMallocAsync, freed on the stream on every return path.
struct AsyncScratch {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    ~AsyncScratch() {
        if (p) cudaFreeAsync(p, s);
    }
};

int prgpu_download_contacts(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* proxies2,
                            uint32_t* bodies2, uint32_t* flags, int32_t* meta2, float* head4, float* pts8,
                            uint32_t* features2) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const uint32_t n = w->h_cnt->n_live;
    if (n_out) *n_out = n;
    if (n > capacity) return fail(w, PRGPU_ECAPACITY, "%u contacts exceed capacity %u", n, capacity);
    if (n == 0) return PRGPU_OK;
    // gather into one device scratch block, then copy out
    const size_t per = 2 + 2 + 1 + 2 + 4 + 8 + 2;  // 32-bit words per contact
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, per * 4 * (size_t)n, w->stream));
    // 16-byte records first so every float4 store is aligned
    float* g_hd = static_cast<float*>(scratch.p);
    float* g_pt = g_hd + 4 * (size_t)n;
    uint32_t* g_pr = reinterpret_cast<uint32_t*>(g_pt + 8 * (size_t)n);
    uint32_t* g_bd = g_pr + 2 * (size_t)n;
    uint32_t* g_fl = g_bd + 2 * (size_t)n;
    int32_t* g_me = reinterpret_cast<int32_t*>(g_fl + n);
    uint32_t* g_ft = reinterpret_cast<uint32_t*>(g_me + 2 * (size_t)n);
    k_gather_contacts<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, n, g_pr, g_bd, g_fl, g_me, g_hd, g_pt, g_ft);
    CU(cudaGetLastError());
    if (proxies2) CU(cudaMemcpyAsync(proxies2, g_pr, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (bodies2) CU(cudaMemcpyAsync(bodies2, g_bd, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (flags) CU(cudaMemcpyAsync(flags, g_fl, 4 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (meta2) CU(cudaMemcpyAsync(meta2, g_me, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (head4) CU(cudaMemcpyAsync(head4, g_hd, 16 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (pts8) CU(cudaMemcpyAsync(pts8, g_pt, 32 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (features2) CU(cudaMemcpyAsync(features2, g_ft, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_query_aabbs(prgpu_world* w, uint32_t n, const uint32_t* worlds, const float* aabb4, uint32_t capacity,
                      uint32_t* counts, uint32_t* shapes) {
    if (!w || (n && (!worlds || !aabb4 || !counts))) return PRGPU_EINVAL;
    for (uint32_t k = 0; k < n; ++k)
        if (worlds[k] >= w->d.n_worlds) return fail(w, PRGPU_EINVAL, "world %u out of range", worlds[k]);
    CU(cudaSetDevice(w->device));
    // The first step creates the proxies; before it the tree is empty (no overlaps).
    if (n == 0 || !w->stepped) {
        for (uint32_t k = 0; k < n; ++k) counts[k] = 0;
        return PRGPU_OK;
    }
    const size_t cap = shapes ? capacity : 0;
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, 16 * (size_t)n + 4 * (size_t)n * (2 + cap) + 16, w->stream));
    float4* g_box = static_cast<float4*>(scratch.p);
    uint32_t* g_world = reinterpret_cast<uint32_t*>(g_box + n);
    uint32_t* g_count = g_world + n;
    uint32_t* g_status = g_count + n;
    uint32_t* g_out = g_status + 1;
    CU(cudaMemcpyAsync(g_box, aabb4, 16 * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(g_world, worlds, 4 * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemsetAsync(g_status, 0, 4, w->stream));
    launch_query_boxes(w->d, w->L, n, g_world, g_box, (uint32_t)cap, g_count, g_out, g_status, w->stream);
    CU(cudaGetLastError());
    uint32_t status = 0;
    CU(cudaMemcpyAsync(counts, g_count, 4 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaMemcpyAsync(&status, g_status, 4, cudaMemcpyDeviceToHost, w->stream));
    if (cap) CU(cudaMemcpyAsync(shapes, g_out, 4 * (size_t)n * cap, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    if (status) return fail(w, PRGPU_ESTATE, "tree walk deeper than its stack");
    bool over = false;
    for (uint32_t k = 0; k < n; ++k) {
        if (counts[k] > cap) { over = over || shapes != nullptr; continue; }
        if (cap) std::sort(shapes + (size_t)k * cap, shapes + (size_t)k * cap + counts[k]);
    }
    if (over) return fail(w, PRGPU_ECAPACITY, "overlaps exceed capacity %u", capacity);
    return PRGPU_OK;
}

int prgpu_query_aabb(prgpu_world* w, uint32_t world, const float* aabb4, uint32_t capacity, uint32_t* n_out,
                     uint32_t* shapes) {
    if (!w || !aabb4) return PRGPU_EINVAL;
    uint32_t count = 0;
    const int rc = prgpu_query_aabbs(w, 1, &world, aabb4, capacity, &count, shapes);
    if (n_out) *n_out = count;
    return rc;
}

int prgpu_raycast(prgpu_world* w, uint32_t n, const uint32_t* worlds, const float* rays5, int32_t* shapes,
                  float* hits5) {
    if (!w || (n && (!worlds || !rays5 || !shapes || !hits5))) return PRGPU_EINVAL;
    for (uint32_t k = 0; k < n; ++k)
        if (worlds[k] >= w->d.n_worlds) return fail(w, PRGPU_EINVAL, "world %u out of range", worlds[k]);
    CU(cudaSetDevice(w->device));
    if (n == 0) return PRGPU_OK;
    if (!w->stepped) {
        for (uint32_t k = 0; k < n; ++k) {
            shapes[k] = -1;
            for (int q = 0; q < 5; ++q) hits5[5 * (size_t)k + q] = 0.f;
        }
        return PRGPU_OK;
    }
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, 48 * (size_t)n + 16, w->stream));
    float* g_ray = static_cast<float*>(scratch.p);
    float* g_hit = g_ray + 5 * (size_t)n;
    uint32_t* g_world = reinterpret_cast<uint32_t*>(g_hit + 5 * (size_t)n);
    int32_t* g_shape = reinterpret_cast<int32_t*>(g_world + n);
    uint32_t* g_status = reinterpret_cast<uint32_t*>(g_shape + n);
    CU(cudaMemcpyAsync(g_ray, rays5, 20 * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(g_world, worlds, 4 * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemsetAsync(g_status, 0, 4, w->stream));
    launch_ray_nearest(w->d, w->L, n, g_world, g_ray, g_shape, g_hit, g_status, w->stream);
    CU(cudaGetLastError());
    uint32_t status = 0;
    CU(cudaMemcpyAsync(shapes, g_shape, 4 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaMemcpyAsync(hits5, g_hit, 20 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaMemcpyAsync(&status, g_status, 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    if (status) return fail(w, PRGPU_ESTATE, "tree walk deeper than its stack");
    return PRGPU_OK;
}

int prgpu_raycast_all(prgpu_world* w, uint32_t world, const float* ray5, uint32_t capacity, uint32_t* n_out,
                      int32_t* shapes, float* hits5) {
    if (!w || !ray5 || !n_out) return PRGPU_EINVAL;
    if (world >= w->d.n_worlds) return fail(w, PRGPU_EINVAL, "world %u out of range", world);
    CU(cudaSetDevice(w->device));
    *n_out = 0;
    if (!w->stepped) return PRGPU_OK;
    const size_t cap = (shapes && hits5) ? capacity : 0;
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, 24 * cap + 16, w->stream));
    float* g_hit = static_cast<float*>(scratch.p);
    int32_t* g_shape = reinterpret_cast<int32_t*>(g_hit + 5 * cap);
    uint32_t* g_count = reinterpret_cast<uint32_t*>(g_shape + cap);
    uint32_t* g_status = g_count + 1;
    CU(cudaMemsetAsync(g_status, 0, 4, w->stream));
    launch_ray_all(w->d, world, ray5, (uint32_t)cap, g_count, g_shape, g_hit, g_status, w->stream);
    CU(cudaGetLastError());
    uint32_t cs[2] = {0u, 0u};
    CU(cudaMemcpyAsync(cs, g_count, 8, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const uint32_t found = cs[0];
    *n_out = found;
    if (cs[1]) {
        CU(cudaFreeAsync(scratch.p, w->stream));
        scratch.p = nullptr;
        return fail(w, PRGPU_ESTATE, "tree walk deeper than its stack");
    }
    const size_t m = std::min<size_t>(found, cap);
    if (m) {
        CU(cudaMemcpyAsync(shapes, g_shape, 4 * m, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaMemcpyAsync(hits5, g_hit, 20 * m, cudaMemcpyDeviceToHost, w->stream));
    }
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    if (found > cap && cap) return fail(w, PRGPU_ECAPACITY, "%u hits exceed capacity %u", found, capacity);
    // in shape order (the reference reports them in tree order)
    std::vector<std::pair<int32_t, uint32_t>> order(m);
    for (size_t k = 0; k < m; ++k) order[k] = {shapes[k], (uint32_t)k};
    std::sort(order.begin(), order.end());
    std::vector<float> h(hits5, hits5 + 5 * m);
    for (size_t k = 0; k < m; ++k) {
        shapes[k] = order[k].first;
        for (int q = 0; q < 5; ++q) hits5[5 * k + q] = h[5 * (size_t)order[k].second + q];
    }
    return PRGPU_OK;
}

int prgpu_download_contact_state(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* slots, float* mat4) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const uint32_t n = w->h_cnt->n_live;
    if (n_out) *n_out = n;
    if (n == 0 || (!slots && !mat4)) return PRGPU_OK;
    if (n > capacity) return fail(w, PRGPU_ECAPACITY, "%u contacts exceed capacity %u", n, capacity);
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, 20 * (size_t)n, w->stream));
    float4* g_mat = static_cast<float4*>(scratch.p);
    uint32_t* g_slot = reinterpret_cast<uint32_t*>(g_mat + n);
    k_gather_contact_state<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, n, g_slot, g_mat);
    CU(cudaGetLastError());
    if (slots) CU(cudaMemcpyAsync(slots, g_slot, 4 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (mat4) CU(cudaMemcpyAsync(mat4, g_mat, 16 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_set_solve_records(prgpu_world* w, int enabled) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    const bool on = enabled != 0;
    if (on == (w->d.cs_post_tag != nullptr)) return PRGPU_OK;
    int rc = drop_graph(w);
    if (rc) return rc;
    if (on) {
        const size_t C = std::max<uint32_t>(w->d.contact_cap, 1);
        if (!w->post_imp) {
            CU(cudaMalloc(&w->post_imp, sizeof(float4) * C));
            CU(cudaMalloc(&w->post_tag, sizeof(uint2) * C));
            CU(cudaMemsetAsync(w->post_tag, 0, sizeof(uint2) * C, w->stream));
        }
        w->d.cs_post = w->post_imp;
        w->d.cs_post_tag = w->post_tag;
    } else {
        w->d.cs_post = nullptr;
        w->d.cs_post_tag = nullptr;
    }
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_download_solve_records(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* slots, uint32_t* info,
                                 float* imp4) {
    if (!w || !n_out) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const uint32_t n = w->h_cnt->n_live;
    *n_out = 0;
    if (n == 0) return PRGPU_OK;
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, 28 * (size_t)n + 16, w->stream));
    float4* g_imp = static_cast<float4*>(scratch.p);
    uint32_t* g_slot = reinterpret_cast<uint32_t*>(g_imp + n);
    uint32_t* g_info = g_slot + n;
    uint32_t* g_n = g_info + n;
    CU(cudaMemsetAsync(g_n, 0, 4, w->stream));
    k_gather_solve_records<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, n, n, g_n, g_slot, g_info, g_imp);
    CU(cudaGetLastError());
    uint32_t m = 0;
    CU(cudaMemcpyAsync(&m, g_n, 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    *n_out = m;
    if (m > capacity && (slots || info || imp4)) return fail(w, PRGPU_ECAPACITY, "%u records exceed capacity %u", m, capacity);
    if (slots) CU(cudaMemcpyAsync(slots, g_slot, 4 * (size_t)m, cudaMemcpyDeviceToHost, w->stream));
    if (info) CU(cudaMemcpyAsync(info, g_info, 4 * (size_t)m, cudaMemcpyDeviceToHost, w->stream));
    if (imp4) CU(cudaMemcpyAsync(imp4, g_imp, 16 * (size_t)m, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_set_contact(prgpu_world* w, uint32_t slot, int enabled, float friction, float restitution,
                      float tangent_speed) {
    if (!w) return PRGPU_EINVAL;
    if (slot >= w->d.contact_cap) return fail(w, PRGPU_EINVAL, "contact slot %u out of range", slot);
    CU(cudaSetDevice(w->device));
    uint32_t* status = reinterpret_cast<uint32_t*>(w->d_stage);
    k_set_contact<<<1, 1, 0, w->stream>>>(w->d, slot, enabled, friction, restitution, tangent_speed, status);
    CU(cudaGetLastError());
    uint32_t st = 0;
    CU(cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (st) return fail(w, PRGPU_EINVAL, "contact slot %u holds no live contact", slot);
    return PRGPU_OK;
}

int prgpu_set_manifold(prgpu_world* w, uint32_t slot, int32_t type, int32_t count, const float* head4,
                       const float* pts8) {
    if (!w || !head4 || !pts8) return PRGPU_EINVAL;
    if (slot >= w->d.contact_cap) return fail(w, PRGPU_EINVAL, "contact slot %u out of range", slot);
    CU(cudaSetDevice(w->device));
    uint32_t* status = reinterpret_cast<uint32_t*>(w->d_stage);
    k_set_manifold<<<1, 1, 0, w->stream>>>(w->d, slot, type, count, make_float4(head4[0], head4[1], head4[2], head4[3]),
                                           make_float4(pts8[0], pts8[1], pts8[2], pts8[3]),
                                           make_float4(pts8[4], pts8[5], pts8[6], pts8[7]), status);
    CU(cudaGetLastError());
    uint32_t st = 0;
    CU(cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (st == 1u) return fail(w, PRGPU_EINVAL, "contact slot %u holds no live contact", slot);
    if (st == 2u) return fail(w, PRGPU_EINVAL, "cannot change the manifold's type or point count");
    return PRGPU_OK;
}

int prgpu_download_contact_seq(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint64_t* seq) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const uint32_t n = w->h_cnt->n_live;
    if (n_out) *n_out = n;
    if (n > capacity) return fail(w, PRGPU_ECAPACITY, "%u contacts exceed capacity %u", n, capacity);
    if (n == 0 || !seq) return PRGPU_OK;
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, 8 * (size_t)n, w->stream));
    uint64_t* g = static_cast<uint64_t*>(scratch.p);
    k_gather_seq<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, n, g);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(seq, g, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

__global__ void k_gather_sweep_order(DW d, uint32_t n, int32_t* items3) {
    GRID_LOOP(t, n) {
        const uint32_t id = d.t_id[t];
        int32_t* o = items3 + 3 * (size_t)t;
        if (id & kJointBit) {
            o[0] = 1; o[1] = (int32_t)(id & ~kJointBit); o[2] = 0;
        } else {
            const uint2 pr = d.cs_proxy[id];
            o[0] = 0; o[1] = (int32_t)min(pr.x, pr.y); o[2] = (int32_t)max(pr.x, pr.y);
        }
    }
}

int prgpu_download_sweep_order(prgpu_world* w, uint32_t capacity, uint32_t* n_out, int32_t* items3) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const uint32_t n = w->stepped ? w->h_cnt->n_active : 0u;
    if (n_out) *n_out = n;
    if (n == 0 || !items3) return PRGPU_OK;  // a count-only call
    if (n > capacity) return fail(w, PRGPU_ECAPACITY, "%u constraints exceed capacity %u", n, capacity);
    AsyncScratch scratch{nullptr, w->stream};
    CU(cudaMallocAsync(&scratch.p, 12 * (size_t)n, w->stream));
    int32_t* g = static_cast<int32_t*>(scratch.p);
    k_gather_sweep_order<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, n, g);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(items3, g, 12 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaFreeAsync(scratch.p, w->stream));
    scratch.p = nullptr;
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

// ---- contact download without device allocation ---------------------------
// Some callers must not allocate device memory once they are running: a
// real-time control or rendering loop that forbids allocation in its steady
// state, or a process whose device memory is held by another framework's
// caching allocator, where a new cudaMalloc/cudaMallocAsync can fail or stall.
// For them prgpu_download_contacts_noalloc gathers into a fixed array in device
// memory that exists from the moment the library is loaded (every GPU that
// loads the library holds it until the process exits).
constexpr uint32_t kNoAllocMaxContacts = 65536;
constexpr size_t kNoAllocWords = 21;  // head 4 + points 8 + proxies 2 + bodies 2 + flags 1 + meta 2 + features 2
static __device__ __align__(256) uint32_t g_noalloc_contacts[kNoAllocMaxContacts * kNoAllocWords];

namespace {
// Device address of g_noalloc_contacts per device.  In host code the array's
// name is only a host-side stand-in, so the address is looked up once per
// device, with that device current, and passed to the gather kernel.
std::mutex g_noalloc_mutex;
uint32_t* g_noalloc_ptr[64] = {};

int noalloc_scratch(prgpu_world* w, uint32_t** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (w->device < 0 || w->device >= 64) return fail(w, PRGPU_EINVAL, "device ordinal out of range");
    if (!g_noalloc_ptr[w->device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_contacts);
        if (e != cudaSuccess || !p)
            return fail(w, PRGPU_ECUDA, "cudaGetSymbolAddress(g_noalloc_contacts): %s", cudaGetErrorString(e));
        g_noalloc_ptr[w->device] = static_cast<uint32_t*>(p);
    }
    *out = g_noalloc_ptr[w->device];
    return PRGPU_OK;
}
}  // namespace

int prgpu_download_contacts_noalloc(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* proxies2,
                                    uint32_t* bodies2, uint32_t* flags, int32_t* meta2, float* head4, float* pts8,
                                    uint32_t* features2) {
    if (!w) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    uint32_t* scratch = nullptr;
    int rc = noalloc_scratch(w, &scratch);
    if (rc) return rc;
    CU(cudaMemcpyAsync(w->h_cnt, w->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const uint32_t n = w->h_cnt->n_live;
    if (n_out) *n_out = n;
    if (n > capacity) return fail(w, PRGPU_ECAPACITY, "%u contacts exceed capacity %u", n, capacity);
    if (n > kNoAllocMaxContacts)
        return fail(w, PRGPU_ECAPACITY,
                    "%u contacts exceed the %u that prgpu_download_contacts_noalloc can stage; "
                    "use prgpu_download_contacts", n, kNoAllocMaxContacts);
    if (n == 0) return PRGPU_OK;
    // The gather writes every word of the n records, so nothing needs clearing.
    float* g_hd = reinterpret_cast<float*>(scratch);
    float* g_pt = g_hd + 4 * (size_t)n;
    uint32_t* g_pr = reinterpret_cast<uint32_t*>(g_pt + 8 * (size_t)n);
    uint32_t* g_bd = g_pr + 2 * (size_t)n;
    uint32_t* g_fl = g_bd + 2 * (size_t)n;
    int32_t* g_me = reinterpret_cast<int32_t*>(g_fl + n);
    uint32_t* g_ft = reinterpret_cast<uint32_t*>(g_me + 2 * (size_t)n);
    k_gather_contacts<<<w->L.grid, w->L.threads, 0, w->stream>>>(w->d, n, g_pr, g_bd, g_fl, g_me, g_hd, g_pt, g_ft);
    CU(cudaGetLastError());
    if (proxies2) CU(cudaMemcpyAsync(proxies2, g_pr, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (bodies2) CU(cudaMemcpyAsync(bodies2, g_bd, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (flags) CU(cudaMemcpyAsync(flags, g_fl, 4 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (meta2) CU(cudaMemcpyAsync(meta2, g_me, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (head4) CU(cudaMemcpyAsync(head4, g_hd, 16 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (pts8) CU(cudaMemcpyAsync(pts8, g_pt, 32 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    if (features2) CU(cudaMemcpyAsync(features2, g_ft, 8 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_download_proxies(prgpu_world* w, float* aabb4) {
    if (!w || !aabb4) return PRGPU_EINVAL;
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(aabb4, w->d.p_aabb, sizeof(float4) * w->d.n_shapes, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_last_error(prgpu_world* w, char* buf, int len) {
    if (!buf || len <= 0) return PRGPU_EINVAL;
    const std::string& e = w ? w->err : std::string();
    std::snprintf(buf, (size_t)len, "%s", e.c_str());
    return PRGPU_OK;
}

// ---- StepAdjoint ---------------------------------------------------------------------
// A window of recorded steps: snapshots of the whole device state every k steps,
// the tapes of one segment at a time, and the adjoint and tangent state.
struct AdjWindow {
    int every = 1;
    int steps = 0;
    prgpu_step_conf conf{};
    bool conf_set = false;
    std::vector<void*> snaps;       // device copies of every allocation, one per checkpoint
    void* end_state = nullptr;
    size_t snap_bytes = 0;
    std::vector<StepTape> tapes;    // host copies of the device structs
    StepTape* d_tapes = nullptr;
    std::vector<std::pair<void*, size_t>> mem;  // tape, adjoint and tangent arrays
    AdjState adj{};
    TanState tan{};
    double* fdot = nullptr;
    float* tgval = nullptr;
    uint32_t kcap = 0, ccap = 0;
    int grid = 0;
    uint32_t mismatches = 0, overflows = 0;
    double forward_ms = 0, record_ms = 0, reverse_ms = 0;  // host time of the phases of the last passes
    std::vector<cudaGraphExec_t> rec_graphs;  // recorded step into tape i, captured once per window
    // steps [taped_lo, taped_hi) of a segment that the forward pass recorded into
    // tapes 0.. as it ran them (its last segment); -1: none
    int taped_lo = -1, taped_hi = -1;
};

void adjoint_drop_graphs(prgpu_world* w) {
    if (!w || !w->adj) return;
    for (cudaGraphExec_t& g : w->adj->rec_graphs)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

// Device memory of closed adjoint windows, (device, size) -> buffer, kept for the
// next window of the same shape (a window allocates its checkpoints, tapes and
// adjoint state up front; re-mapping gigabytes every window would cost more than
// the window's steps).  prgpu_adjoint_trim frees it.
static std::mutex g_adj_cache_mu;
static std::multimap<std::pair<int, size_t>, void*> g_adj_cache;

static void adj_give(const prgpu_world* w, void* p, size_t bytes) {
    std::lock_guard<std::mutex> lk(g_adj_cache_mu);
    g_adj_cache.emplace(std::make_pair(w->device, bytes), p);
}

// A buffer of exactly `bytes` from the cache, else a new one.
static cudaError_t adj_take(prgpu_world* w, void** p, size_t bytes) {
    {
        std::lock_guard<std::mutex> lk(g_adj_cache_mu);
        auto it = g_adj_cache.find(std::make_pair(w->device, bytes));
        if (it != g_adj_cache.end()) {
            *p = it->second;
            g_adj_cache.erase(it);
            return cudaSuccess;
        }
    }
    return cudaMalloc(p, bytes);
}

static int adj_alloc(prgpu_world* w, AdjWindow* a, void** p, size_t bytes) {
    *p = nullptr;
    bytes = std::max<size_t>(bytes, 16);
    const cudaError_t e = adj_take(w, p, bytes);
    if (e != cudaSuccess) return fail(w, PRGPU_ECUDA, "adjoint cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    a->mem.push_back({*p, bytes});
    return PRGPU_OK;
}

void adjoint_close(prgpu_world* w) {
    if (!w || !w->adj) return;
    AdjWindow* a = w->adj;
    cudaStreamSynchronize(w->stream);
    adjoint_drop_graphs(w);
    for (void* p : a->snaps) adj_give(w, p, a->snap_bytes);
    if (a->end_state) adj_give(w, a->end_state, a->snap_bytes);
    for (const auto& m : a->mem) adj_give(w, m.first, m.second);
    delete a;
    w->adj = nullptr;
    w->d.tape = nullptr;
}

static int snap_copy(prgpu_world* w, void* buf, bool save) {
    size_t off = 0;
    for (size_t i = 0; i < w->allocs.size(); ++i) {
        if (w->alloc_scratch[i]) continue;
        char* b = static_cast<char*>(buf) + off;
        const cudaError_t e = save ? cudaMemcpyAsync(b, w->allocs[i], w->alloc_bytes[i], cudaMemcpyDeviceToDevice, w->stream)
                                   : cudaMemcpyAsync(w->allocs[i], b, w->alloc_bytes[i], cudaMemcpyDeviceToDevice, w->stream);
        if (e != cudaSuccess) return fail(w, PRGPU_ECUDA, "snapshot copy: %s", cudaGetErrorString(e));
        off += (w->alloc_bytes[i] + 255) & ~(size_t)255;
    }
    return PRGPU_OK;
}

static size_t snap_size(const prgpu_world* w) {
    size_t t = 0;
    for (size_t i = 0; i < w->allocs.size(); ++i)
        if (!w->alloc_scratch[i]) t += (w->alloc_bytes[i] + 255) & ~(size_t)255;
    return t;
}

// Re-runs the steps [first, first + n) of the window from their checkpoint
// with recording on, one tape per step (grid-wide solve, same results).
// Counts words that differ between two device arrays.
__global__ void k_count_diff(const uint32_t* a, const uint32_t* b, size_t n, uint32_t* out) {
    uint32_t c = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        c += (a[i] != b[i]) ? 1u : 0u;
    if (c) atomicAdd(out, c);
}

// Byte offset of a world allocation inside a snapshot.
static size_t snap_offset(const prgpu_world* w, const void* p) {
    size_t off = 0;
    for (size_t i = 0; i < w->allocs.size(); ++i) {
        if (w->alloc_scratch[i]) continue;
        if (w->allocs[i] == p) return off;
        off += (w->alloc_bytes[i] + 255) & ~(size_t)255;
    }
    return (size_t)-1;
}

// Whether the live positions and velocities equal those in snapshot `snap`
// (a re-recorded segment must end where the forward pass went on from).
static int check_against(prgpu_world* w, const void* snap, uint32_t* differ) {
    AdjWindow* a = w->adj;
    CU(cudaMemsetAsync(a->adj.err + 1, 0, sizeof(uint32_t), w->stream));
    const size_t N4 = 4 * (size_t)w->d.n_bodies;
    for (const void* p : {(const void*)w->d.b_pos1, (const void*)w->d.b_vel}) {
        const size_t off = snap_offset(w, p);
        if (off == (size_t)-1) return fail(w, PRGPU_ESTATE, "snapshot layout");
        k_count_diff<<<64, 256, 0, w->stream>>>(static_cast<const uint32_t*>(p),
                                                reinterpret_cast<const uint32_t*>(static_cast<const char*>(snap) + off),
                                                N4, a->adj.err + 1);
    }
    CU(cudaMemcpyAsync(differ, a->adj.err + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

// Captures one recorded step into tape i: the tape's per-step words reset, then
// the regular step with d.tape set, in the per-world sweep layout that the
// adjoint and tangent kernels follow.
static int capture_record_step(prgpu_world* w, int i) {
    AdjWindow* a = w->adj;
    const StepTape& t = a->tapes[i];
    const bool per_world = w->L.per_world;
    CU(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(t.src, 0xfe, 2 * (size_t)a->ccap, w->stream);
    cudaMemsetAsync(t.created, 0, a->ccap, w->stream);
    cudaMemsetAsync(t.hdr, 0, sizeof(uint32_t) * (kSerialColour + 6), w->stream);
    w->L.per_world = true;
    w->d.tape = a->d_tapes + i;
    enqueue_step(w, true, nullptr, true);
    w->d.tape = nullptr;
    w->L.per_world = per_world;
    cudaGraph_t g = nullptr;
    const cudaError_t e1 = cudaStreamEndCapture(w->stream, &g);
    if (e1 != cudaSuccess) return fail(w, PRGPU_ECUDA, "record capture: %s", cudaGetErrorString(e1));
    const cudaError_t e2 = cudaGraphInstantiate(&a->rec_graphs[i], g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) {
        a->rec_graphs[i] = nullptr;
        return fail(w, PRGPU_ECUDA, "record instantiate: %s", cudaGetErrorString(e2));
    }
    return PRGPU_OK;
}

// One step recorded into tape i (the window's configuration already uploaded).
static int record_step(prgpu_world* w, int i) {
    AdjWindow* a = w->adj;
    a->rec_graphs.resize(a->every, nullptr);
    int rc = 0;
    if (!a->rec_graphs[i] && (rc = capture_record_step(w, i))) return rc;
    CU(cudaGraphLaunch(a->rec_graphs[i], w->stream));
    return PRGPU_OK;
}

// Adds the replay mismatches of the differentiable restatement recorded in
// tapes 0..n-1, then checks the device error word.
static int count_tape_mismatches(prgpu_world* w, int n) {
    AdjWindow* a = w->adj;
    std::vector<uint32_t> bad(n, 0);
    for (int i = 0; i < n; ++i)
        CU(cudaMemcpyAsync(&bad[i], a->tapes[i].hdr + kSerialColour + 5, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    for (int i = 0; i < n; ++i) a->mismatches += bad[i];
    return check_device_error(w);
}

static int record_segment(prgpu_world* w, int seg, int n) {
    AdjWindow* a = w->adj;
    int rc = snap_copy(w, a->snaps[seg], false);
    if (rc) return rc;
    // the checkpoint holds the configuration of the step before it: upload the window's
    w->conf_valid = false;
    rc = set_conf(w, &a->conf);
    if (rc) return rc;
    for (int i = 0; i < n; ++i)
        if ((rc = record_step(w, i))) return rc;
    if ((rc = count_tape_mismatches(w, n))) return rc;
    // the segment must end where the forward pass continued from
    const void* next = (size_t)(seg + 1) < a->snaps.size() ? a->snaps[seg + 1] : a->end_state;
    uint32_t differ = 0;
    if (next && (rc = check_against(w, next, &differ))) return rc;
    a->mismatches += differ;
    return PRGPU_OK;
}

int prgpu_adjoint_begin(prgpu_world* w, int checkpoint_every) {
    if (!w || checkpoint_every < 1) return PRGPU_EINVAL;
    if (w->adj) return fail(w, PRGPU_ESTATE, "an adjoint window is already open");
    CU(cudaSetDevice(w->device));
    if (w->d.n_joints) {  // the differentiated joint is the revolute point constraint
        std::vector<uint32_t> jf(w->d.n_joints);
        CU(cudaMemcpy(jf.data(), w->d.j_flags, sizeof(uint32_t) * jf.size(), cudaMemcpyDeviceToHost));
        for (uint32_t f : jf)
            if ((f & 3u) || (f >> 8))
                return fail(w, PRGPU_EINVAL, "adjoint: only revolute joints without a limit or a motor are differentiated");
    }
    AdjWindow* a = new AdjWindow();
    a->every = checkpoint_every;
    a->kcap = w->d.contact_cap + w->d.n_joints;
    a->ccap = w->d.contact_cap;
    a->snap_bytes = snap_size(w);
    a->grid = (int)adj_parallel_grid();
    w->adj = a;
    if (a->grid < 1) { adjoint_close(w); return fail(w, PRGPU_ECUDA, "adjoint: no device"); }
    const uint32_t N = w->d.n_bodies, K = a->kcap, C = a->ccap, S = w->d.n_shapes;
    int rc = 0;
#define AA(ptr, bytes) do { void* q_; rc = adj_alloc(w, a, &q_, (bytes)); if (rc) { adjoint_close(w); return rc; } \
                            ptr = reinterpret_cast<decltype(ptr)>(q_); } while (0)
    AA(a->adj.pbar, sizeof(float4) * N); AA(a->adj.vbar, sizeof(float4) * N); AA(a->adj.vibar, sizeof(float4) * N);
    AA(a->adj.vi, sizeof(float4) * N); AA(a->adj.lbar, sizeof(float4) * K); AA(a->adj.pvacc, sizeof(double) * 6 * N);
    AA(a->adj.gbar, sizeof(float) * kAdjGeomWords * (size_t)K); AA(a->adj.gval, sizeof(float) * kAdjGeomWords * (size_t)K);
    AA(a->adj.mbar, sizeof(float4) * C); AA(a->adj.mtmp, sizeof(float4) * C); AA(a->adj.fbar, sizeof(float) * S);
    AA(a->adj.err, sizeof(uint32_t) * 2);
    AA(a->adj.jbar, sizeof(float4) * std::max<uint32_t>(w->d.n_joints, 1));
    a->adj.grid = (uint32_t)a->grid;
    // one block per world in the reverse sweeps; larger worlds get larger blocks
    const uint32_t most = w->order_nb.empty() ? 0u : *std::max_element(w->order_nb.begin(), w->order_nb.end());
    a->adj.sweep_threads = adj_sweep_threads(most, w->d.n_worlds);
    AA(a->tan.jdot, sizeof(double) * 2 * std::max<uint32_t>(w->d.n_joints, 1));
    AA(a->tan.pdot, sizeof(double) * 3 * N); AA(a->tan.vdot, sizeof(double) * 3 * N);
    AA(a->tan.vidot, sizeof(double) * 3 * N); AA(a->tan.ldot, sizeof(double) * 4 * (size_t)K);
    AA(a->tan.gdot, sizeof(double) * kAdjGeomWords * (size_t)K); AA(a->tan.mdot, sizeof(double) * 4 * (size_t)C);
    AA(a->tan.mtmp, sizeof(double) * 4 * (size_t)C); AA(a->fdot, sizeof(double) * S);
    a->tan.fdot = a->fdot;
    AA(a->tgval, sizeof(float) * kAdjGeomWords * (size_t)K);
    return PRGPU_OK;
}

static int ensure_tapes(prgpu_world* w) {
    AdjWindow* a = w->adj;
    if (!a->tapes.empty()) return PRGPU_OK;
    const uint32_t N = w->d.n_bodies, K = a->kcap, C = a->ccap;
    const int iv = std::max(0, a->conf.regVelocityIters), ip = std::min(std::max(0, a->conf.regPositionIters), kMaxPosIters);
    a->tapes.resize(a->every);
    int rc = 0;
    for (int i = 0; i < a->every; ++i) {
        StepTape& t = a->tapes[i];
        t.iv = iv; t.ip = ip; t.kcap = K;
        AA(t.p0, sizeof(float4) * N); AA(t.v0, sizeof(float4) * N); AA(t.flags, sizeof(uint32_t) * N);
        AA(t.slept, N); AA(t.t_id, sizeof(uint32_t) * K); AA(t.pc, sizeof(PC) * K); AA(t.cinfo, sizeof(float4) * K);
        AA(t.prox, sizeof(uint2) * K); AA(t.imp0, sizeof(float4) * K); AA(t.warm, sizeof(float4) * 2 * (size_t)K);
        AA(t.vel, sizeof(float4) * 3 * (size_t)K * std::max(iv, 1));
        AA(t.pos, sizeof(float4) * 2 * (size_t)K * std::max(ip, 1));
        AA(t.src, 2 * (size_t)C); AA(t.created, C); AA(t.hdr, sizeof(uint32_t) * (kSerialColour + 6));
        AA(t.wseg, sizeof(uint32_t) * 2 * (size_t)w->d.n_worlds);
        AA(t.wcol, sizeof(uint32_t) * kColStride * (size_t)w->d.n_worlds);
    }
    AA(a->d_tapes, sizeof(StepTape) * a->every);
    CU(cudaMemcpyAsync(a->d_tapes, a->tapes.data(), sizeof(StepTape) * a->every, cudaMemcpyHostToDevice, w->stream));
#undef AA
    return PRGPU_OK;
}

int prgpu_adjoint_forward(prgpu_world* w, const prgpu_step_conf* conf, int n_steps) {
    if (!w || !conf || n_steps < 0) return PRGPU_EINVAL;
    AdjWindow* a = w->adj;
    if (!a) return fail(w, PRGPU_ESTATE, "no adjoint window is open");
    if (conf->deltaTime == 0.f) return fail(w, PRGPU_EINVAL, "adjoint steps need deltaTime > 0");
    if (conf->doToi) return fail(w, PRGPU_EINVAL, "the adjoint differentiates the regular phase: doToi must be 0");
    if (a->conf_set && std::memcmp(&a->conf, conf, sizeof(*conf)) != 0)
        return fail(w, PRGPU_EINVAL, "one step configuration per adjoint window");
    a->conf = *conf;
    a->conf_set = true;
    CU(cudaSetDevice(w->device));
    int rc = ensure_tapes(w);
    if (rc) return rc;
    const auto t0 = std::chrono::steady_clock::now();
    // the window's last segment as of this call is recorded as it runs, so that
    // the backward pass (if it comes next) need not run it again
    const int end = a->steps + n_steps;
    const int tail_first = end > 0 ? ((end - 1) / a->every) * a->every : 0;
    for (int i = 0; i < n_steps; ++i) {
        const int s = a->steps, seg_first = s - s % a->every;
        if (s == seg_first) {
            void* buf = nullptr;
            if (adj_take(w, &buf, a->snap_bytes) != cudaSuccess) return fail(w, PRGPU_ECUDA, "checkpoint allocation");
            a->snaps.push_back(buf);
            if ((rc = snap_copy(w, buf, true))) return rc;
        }
        const bool tape = s >= tail_first && (s == seg_first || (a->taped_lo == seg_first && a->taped_hi == s));
        if (tape) {
            if ((rc = set_conf(w, conf))) return rc;
            w->stepped = true;
            if ((rc = record_step(w, s - seg_first))) return rc;
            if (s == seg_first) a->taped_lo = s;
            a->taped_hi = s + 1;
        } else if ((rc = run_steps(w, conf, 1, false))) {
            return rc;
        }
        ++a->steps;
    }
    rc = check_device_error(w);
    a->forward_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int prgpu_adjoint_profile(prgpu_world* w, double* forward_ms, double* record_ms, double* reverse_ms) {
    if (!w) return PRGPU_EINVAL;
    if (!w->adj) return fail(w, PRGPU_ESTATE, "no adjoint window is open");
    if (forward_ms) *forward_ms = w->adj->forward_ms;
    if (record_ms) *record_ms = w->adj->record_ms;
    if (reverse_ms) *reverse_ms = w->adj->reverse_ms;
    return PRGPU_OK;
}

int prgpu_adjoint_backward(prgpu_world* w, const float* dl_dpos3, const float* dl_dvel3, float* dl_dpos3_start,
                           float* dl_dvel3_start, float* dl_dfriction) {
    if (!w) return PRGPU_EINVAL;
    AdjWindow* a = w->adj;
    if (!a) return fail(w, PRGPU_ESTATE, "no adjoint window is open");
    if (a->steps == 0) return fail(w, PRGPU_ESTATE, "the adjoint window has no steps");
    CU(cudaSetDevice(w->device));
    const uint32_t N = w->d.n_bodies, S = w->d.n_shapes;
    int rc = 0;
    if (!a->end_state && adj_take(w, &a->end_state, a->snap_bytes) != cudaSuccess)
        return fail(w, PRGPU_ECUDA, "end-state allocation");
    if ((rc = snap_copy(w, a->end_state, true))) return rc;
    std::vector<float4> h(N);
    for (uint32_t b = 0; b < N; ++b)
        h[b] = make_float4(dl_dpos3 ? dl_dpos3[3 * b] : 0.f, dl_dpos3 ? dl_dpos3[3 * b + 1] : 0.f,
                           dl_dpos3 ? dl_dpos3[3 * b + 2] : 0.f, 0.f);
    CU(cudaMemcpyAsync(a->adj.pbar, h.data(), sizeof(float4) * N, cudaMemcpyHostToDevice, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    for (uint32_t b = 0; b < N; ++b)
        h[b] = make_float4(dl_dvel3 ? dl_dvel3[3 * b] : 0.f, dl_dvel3 ? dl_dvel3[3 * b + 1] : 0.f,
                           dl_dvel3 ? dl_dvel3[3 * b + 2] : 0.f, 0.f);
    CU(cudaMemcpyAsync(a->adj.vbar, h.data(), sizeof(float4) * N, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemsetAsync(a->adj.mbar, 0, sizeof(float4) * a->ccap, w->stream));
    CU(cudaMemsetAsync(a->adj.pvacc, 0, sizeof(double) * 6 * N, w->stream));
    CU(cudaMemsetAsync(a->adj.jbar, 0, sizeof(float4) * std::max<uint32_t>(w->d.n_joints, 1), w->stream));
    CU(cudaMemsetAsync(a->adj.fbar, 0, sizeof(float) * std::max<uint32_t>(S, 1), w->stream));
    CU(cudaMemsetAsync(a->adj.err, 0, sizeof(uint32_t), w->stream));
    const int nseg = (a->steps + a->every - 1) / a->every;
    using clk = std::chrono::steady_clock;
    a->record_ms = a->reverse_ms = 0;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int first = seg * a->every, n = std::min(a->every, a->steps - first);
        const auto t0 = clk::now();
        if (first == a->taped_lo && a->steps == a->taped_hi) {
            // the forward pass recorded this segment as it ran it; the world is
            // at the segment's end, as a recomputation would leave it
            if ((rc = count_tape_mismatches(w, n))) return rc;
        } else if ((rc = record_segment(w, seg, n))) {
            return rc;
        }
        a->taped_lo = a->taped_hi = -1;  // the tapes now hold other segments
        const auto t1 = clk::now();
        for (int i = n - 1; i >= 0; --i) {
            const cudaError_t e = launch_adj_step(w->d, a->d_tapes + i, a->adj, a->ccap, w->stream);
            if (e != cudaSuccess) return fail(w, PRGPU_ECUDA, "adjoint step: %s", cudaGetErrorString(e));
        }
        if ((rc = check_device_error(w))) return rc;
        const auto t2 = clk::now();
        a->record_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        a->reverse_ms += std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    if ((rc = snap_copy(w, a->end_state, false))) return rc;
    uint32_t err = 0;
    CU(cudaMemcpyAsync(&err, a->adj.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream));
    std::vector<float4> hp(N), hv(N);
    std::vector<uint32_t> fl(N);
    CU(cudaMemcpyAsync(hp.data(), a->adj.pbar, sizeof(float4) * N, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaMemcpyAsync(hv.data(), a->adj.vbar, sizeof(float4) * N, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaMemcpyAsync(fl.data(), w->d.b_flags, sizeof(uint32_t) * N, cudaMemcpyDeviceToHost, w->stream));
    if (dl_dfriction) CU(cudaMemcpyAsync(dl_dfriction, a->adj.fbar, sizeof(float) * S, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    a->overflows += err;
    for (uint32_t b = 0; b < N; ++b) {
        // only dynamic bodies' states are differentiated
        const bool dyn = is_accelerable(fl[b]);
        if (dl_dpos3_start) {
            dl_dpos3_start[3 * b] = dyn ? hp[b].x : 0.f; dl_dpos3_start[3 * b + 1] = dyn ? hp[b].y : 0.f;
            dl_dpos3_start[3 * b + 2] = dyn ? hp[b].z : 0.f;
        }
        if (dl_dvel3_start) {
            dl_dvel3_start[3 * b] = dyn ? hv[b].x : 0.f; dl_dvel3_start[3 * b + 1] = dyn ? hv[b].y : 0.f;
            dl_dvel3_start[3 * b + 2] = dyn ? hv[b].z : 0.f;
        }
    }
    if (err) return fail(w, PRGPU_ECAPACITY, "adjoint: %u local derivative tapes overflowed", err);
    return PRGPU_OK;
}

int prgpu_adjoint_tangent(prgpu_world* w, const double* dpos3_start, const double* dvel3_start, const double* dfriction,
                          double* dpos3_end, double* dvel3_end) {
    if (!w) return PRGPU_EINVAL;
    AdjWindow* a = w->adj;
    if (!a) return fail(w, PRGPU_ESTATE, "no adjoint window is open");
    if (a->steps == 0) return fail(w, PRGPU_ESTATE, "the adjoint window has no steps");
    CU(cudaSetDevice(w->device));
    const uint32_t N = w->d.n_bodies, S = w->d.n_shapes;
    int rc = 0;
    if (!a->end_state && adj_take(w, &a->end_state, a->snap_bytes) != cudaSuccess)
        return fail(w, PRGPU_ECUDA, "end-state allocation");
    if ((rc = snap_copy(w, a->end_state, true))) return rc;
    std::vector<double> z(3 * (size_t)N, 0.0), zf(std::max<uint32_t>(S, 1), 0.0);
    CU(cudaMemcpyAsync(a->tan.pdot, dpos3_start ? dpos3_start : z.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(a->tan.vdot, dvel3_start ? dvel3_start : z.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(a->fdot, dfriction ? dfriction : zf.data(), sizeof(double) * S, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemsetAsync(a->tan.mdot, 0, sizeof(double) * 4 * a->ccap, w->stream));
    CU(cudaMemsetAsync(a->tan.jdot, 0, sizeof(double) * 2 * std::max<uint32_t>(w->d.n_joints, 1), w->stream));
    CU(cudaStreamSynchronize(w->stream));
    const int nseg = (a->steps + a->every - 1) / a->every;
    a->taped_lo = a->taped_hi = -1;  // the segments below are recorded over the tapes
    for (int seg = 0; seg < nseg; ++seg) {
        const int first = seg * a->every, n = std::min(a->every, a->steps - first);
        if ((rc = record_segment(w, seg, n))) return rc;
        for (int i = 0; i < n; ++i) {
            const cudaError_t e = launch_tan_step(w->d, a->d_tapes + i, a->tan, a->tgval, a->ccap, w->stream);
            if (e != cudaSuccess) return fail(w, PRGPU_ECUDA, "tangent step: %s", cudaGetErrorString(e));
        }
        if ((rc = check_device_error(w))) return rc;
    }
    if ((rc = snap_copy(w, a->end_state, false))) return rc;
    if (dpos3_end) CU(cudaMemcpyAsync(dpos3_end, a->tan.pdot, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, w->stream));
    if (dvel3_end) CU(cudaMemcpyAsync(dvel3_end, a->tan.vdot, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PRGPU_OK;
}

int prgpu_adjoint_info(prgpu_world* w, int* steps, uint32_t* replay_mismatches, uint32_t* tape_overflows) {
    if (!w) return PRGPU_EINVAL;
    if (!w->adj) return fail(w, PRGPU_ESTATE, "no adjoint window is open");
    if (steps) *steps = w->adj->steps;
    if (replay_mismatches) *replay_mismatches = w->adj->mismatches;
    if (tape_overflows) *tape_overflows = w->adj->overflows;
    return PRGPU_OK;
}

int prgpu_adjoint_trim(void) {
    std::lock_guard<std::mutex> lk(g_adj_cache_mu);
    int dev = -1;
    cudaGetDevice(&dev);
    for (const auto& m : g_adj_cache) {
        cudaSetDevice(m.first.first);
        cudaFree(m.second);
    }
    g_adj_cache.clear();
    if (dev >= 0) cudaSetDevice(dev);
    return PRGPU_OK;
}

int prgpu_adjoint_end(prgpu_world* w) {
    if (!w) return PRGPU_EINVAL;
    if (!w->adj) return fail(w, PRGPU_ESTATE, "no adjoint window is open");
    cudaSetDevice(w->device);
    cudaStreamSynchronize(w->stream);
    adjoint_close(w);
    return PRGPU_OK;
}

}  // extern "C"
