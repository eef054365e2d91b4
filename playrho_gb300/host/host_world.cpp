// host_world.cpp -- HostWorld: pools, GPU batch construction and state mirroring.
#include "host_world.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace prgpu {

namespace {

template <class T>
uint32_t pool_add(std::vector<T>& pool, std::vector<bool>& live, std::vector<uint32_t>& free_ids, const T& v) {
    if (!free_ids.empty()) {
        const uint32_t id = free_ids.back();
        free_ids.pop_back();
        pool[id] = v;
        live[id] = true;
        return id;
    }
    pool.push_back(v);
    live.push_back(true);
    return (uint32_t)(pool.size() - 1);
}

// Tree leaf ID of the k-th proxy of a tree built without removals: leaf 0 is the
// root (node 0); every later leaf takes a node and its new parent the next
// (DynamicTree::CreateLeaf, DynamicTree.cpp:517-569).
uint32_t leaf_id(uint32_t k) { return k == 0u ? 0u : 2u * k - 1u; }

// Whether b differs from a at most in position and velocity (what the GPU batch
// takes in place); mass fields count only when the body sets its own.
// (cx, cy and under_active_time are outputs and never compared.)
bool same_state_only(const HostBody& a, const HostBody& b) {
    const bool mass_same = !b.explicit_mass ||
                           (a.inv_mass == b.inv_mass && a.inv_rot_inertia == b.inv_rot_inertia && a.lcx == b.lcx &&
                            a.lcy == b.lcy);
    return a.type == b.type && a.ax == b.ax && a.ay == b.ay && a.aa == b.aa &&
           a.linear_damping == b.linear_damping && a.angular_damping == b.angular_damping && a.flags == b.flags &&
           a.explicit_mass == b.explicit_mass && mass_same && a.shapes == b.shapes;
}

}  // namespace

HostWorld::HostWorld(const HostWorld& o)
    : device_(o.device_), bodies_(o.bodies_), shapes_(o.shapes_), joints_(o.joints_), body_live_(o.body_live_),
      shape_live_(o.shape_live_), joint_live_(o.joint_live_), body_free_(o.body_free_), shape_free_(o.shape_free_),
      joint_free_(o.joint_free_) {}

HostWorld& HostWorld::operator=(const HostWorld& o) {
    if (this == &o) return *this;
    Drop();
    device_ = o.device_;
    bodies_ = o.bodies_; shapes_ = o.shapes_; joints_ = o.joints_;
    body_live_ = o.body_live_; shape_live_ = o.shape_live_; joint_live_ = o.joint_live_;
    body_free_ = o.body_free_; shape_free_ = o.shape_free_; joint_free_ = o.joint_free_;
    rebuild_ = true;
    contacts_valid_ = false;
    contacts_.clear();
    return *this;
}

HostWorld::~HostWorld() { Drop(); }

void HostWorld::Drop() {
    if (gpu_) prgpu_world_destroy(gpu_);
    gpu_ = nullptr;
    rebuild_ = true;
}

void HostWorld::Check(int rc, const char* what) const {
    if (rc == PRGPU_OK) return;
    char buf[512] = {0};
    if (gpu_) prgpu_last_error(gpu_, buf, (int)sizeof(buf));
    throw Error(rc, std::string(what) + ": " + (buf[0] ? buf : "status " + std::to_string(rc)));
}

// ---- bodies ------------------------------------------------------------------
uint32_t HostWorld::CreateBody(const HostBody& b) {
    for (uint32_t s : b.shapes)
        if (!ShapeAlive(s)) throw Error(PRGPU_EINVAL, "CreateBody: shape ID out of range");
    const uint32_t id = pool_add(bodies_, body_live_, body_free_, b);
    rebuild_ = true;
    return id;
}

const HostBody& HostWorld::GetBody(uint32_t id) const {
    if (!BodyAlive(id)) throw Error(PRGPU_EINVAL, "GetBody: body ID out of range");
    return bodies_[id];
}

void HostWorld::SetBody(uint32_t id, const HostBody& b) {
    if (!BodyAlive(id)) throw Error(PRGPU_EINVAL, "SetBody: body ID out of range");
    for (uint32_t s : b.shapes)
        if (!ShapeAlive(s)) throw Error(PRGPU_EINVAL, "SetBody: shape ID out of range");
    if (!same_state_only(bodies_[id], b)) {
        rebuild_ = true;
    } else if (b.x != bodies_[id].x || b.y != bodies_[id].y || b.angle != bodies_[id].angle ||
               b.vx != bodies_[id].vx || b.vy != bodies_[id].vy || b.w != bodies_[id].w) {
        if (state_dirty_.size() < bodies_.size()) state_dirty_.resize(bodies_.size(), false);
        state_dirty_[id] = true;
    }
    bodies_[id] = b;
}

void HostWorld::DestroyBody(uint32_t id) {
    if (!BodyAlive(id)) throw Error(PRGPU_EINVAL, "Destroy: body ID out of range");
    // joints of the body go with it (AabbTreeWorld.cpp Destroy(BodyID))
    for (uint32_t j = 0; j < joints_.size(); ++j)
        if (joint_live_[j] && (joints_[j].body_a == id || joints_[j].body_b == id)) DestroyJoint(j);
    body_live_[id] = false;
    bodies_[id] = HostBody{};
    body_free_.push_back(id);
    rebuild_ = true;
}

// ---- shapes ------------------------------------------------------------------
uint32_t HostWorld::CreateShape(const HostShape& s) {
    auto valid = [&](const std::vector<float>& v) {
        const size_t nv = v.size() / 2;
        return !(v.size() % 2 || nv < 1 || nv > 16 || (s.kind == PRGPU_DISK && nv != 1) ||
                 (s.kind == PRGPU_EDGE && nv != 2) || s.kind < PRGPU_DISK || s.kind > PRGPU_EDGE);
    };
    bool ok = s.children.empty() ? valid(s.verts) : s.kind != PRGPU_DISK;
    for (const auto& c : s.children) ok = ok && valid(c);
    if (!ok)
        throw Error(PRGPU_EINVAL, "CreateShape: unsupported shape (disk, polygon of <= 16 vertices, edge, "
                                  "or children of edges or polygons)");
    const uint32_t id = pool_add(shapes_, shape_live_, shape_free_, s);
    rebuild_ = true;
    return id;
}

const HostShape& HostWorld::GetShape(uint32_t id) const {
    if (!ShapeAlive(id)) throw Error(PRGPU_EINVAL, "GetShape: shape ID out of range");
    return shapes_[id];
}

void HostWorld::SetShape(uint32_t id, const HostShape& s) {
    if (!ShapeAlive(id)) throw Error(PRGPU_EINVAL, "SetShape: shape ID out of range");
    shapes_[id] = s;
    rebuild_ = true;
}

void HostWorld::DestroyShape(uint32_t id) {
    if (!ShapeAlive(id)) throw Error(PRGPU_EINVAL, "Destroy: shape ID out of range");
    for (uint32_t b = 0; b < bodies_.size(); ++b) {
        if (!body_live_[b]) continue;
        auto& v = bodies_[b].shapes;
        for (size_t k = 0; k < v.size();)
            if (v[k] == id) v.erase(v.begin() + (long)k); else ++k;
    }
    shape_live_[id] = false;
    shapes_[id] = HostShape{};
    shape_free_.push_back(id);
    rebuild_ = true;
}

// ---- joints ------------------------------------------------------------------
uint32_t HostWorld::CreateJoint(const HostJoint& j) {
    if (!BodyAlive(j.body_a) || !BodyAlive(j.body_b)) throw Error(PRGPU_EINVAL, "CreateJoint: body ID out of range");
    const uint32_t id = pool_add(joints_, joint_live_, joint_free_, j);
    rebuild_ = true;
    return id;
}

const HostJoint& HostWorld::GetJoint(uint32_t id) const {
    if (!JointAlive(id)) throw Error(PRGPU_EINVAL, "GetJoint: joint ID out of range");
    return joints_[id];
}

void HostWorld::SetJoint(uint32_t id, const HostJoint& j) {
    if (!JointAlive(id)) throw Error(PRGPU_EINVAL, "SetJoint: joint ID out of range");
    if (!BodyAlive(j.body_a) || !BodyAlive(j.body_b)) throw Error(PRGPU_EINVAL, "SetJoint: body ID out of range");
    joints_[id] = j;
    rebuild_ = true;
}

void HostWorld::DestroyJoint(uint32_t id) {
    if (!JointAlive(id)) throw Error(PRGPU_EINVAL, "Destroy: joint ID out of range");
    joint_live_[id] = false;
    joints_[id] = HostJoint{};
    joint_free_.push_back(id);
    rebuild_ = true;
}

void HostWorld::Clear() {
    Drop();
    bodies_.clear(); shapes_.clear(); joints_.clear();
    body_live_.clear(); shape_live_.clear(); joint_live_.clear();
    body_free_.clear(); shape_free_.clear(); joint_free_.clear();
    state_dirty_.clear();
    contacts_.clear();
    contacts_valid_ = false;
}

// ---- GPU batch -----------------------------------------------------------------
void HostWorld::Build() {
    const uint32_t NB = (uint32_t)bodies_.size();
    gpu_body_.clear();
    body_gpu_.assign(NB, ~0u);
    for (uint32_t b = 0; b < NB; ++b)
        if (body_live_[b]) { body_gpu_[b] = (uint32_t)gpu_body_.size(); gpu_body_.push_back(b); }
    const uint32_t N = (uint32_t)gpu_body_.size();
    std::vector<int32_t> type(N);
    std::vector<float> pos(3 * N), vel(3 * N), acc(3 * N), damp(2 * N);
    std::vector<uint32_t> flags(N);
    bool any_mass = false;
    for (uint32_t i = 0; i < N; ++i) {
        const HostBody& b = bodies_[gpu_body_[i]];
        type[i] = b.type;
        pos[3 * i] = b.x; pos[3 * i + 1] = b.y; pos[3 * i + 2] = b.angle;
        vel[3 * i] = b.vx; vel[3 * i + 1] = b.vy; vel[3 * i + 2] = b.w;
        acc[3 * i] = b.ax; acc[3 * i + 1] = b.ay; acc[3 * i + 2] = b.aa;
        damp[2 * i] = b.linear_damping; damp[2 * i + 1] = b.angular_damping;
        flags[i] = b.flags;
        any_mass = any_mass || (b.explicit_mass && b.type == PRGPU_DYNAMIC);
    }
    // proxies: every (body, attached shape), bodies in ID order, shapes in attach order
    proxy_body_.clear(); proxy_shape_.clear(); proxy_child_.clear();
    std::vector<uint32_t> s_body, s_voff, s_nv;
    std::vector<int32_t> s_kind, s_filter, s_owner;
    bool any_children = false;
    std::vector<float> s_radius, s_density, s_friction, s_restitution, verts;
    for (uint32_t i = 0; i < N; ++i) {
        for (uint32_t sid : bodies_[gpu_body_[i]].shapes) {
            const HostShape& s = shapes_[sid];
            const size_t nc = s.children.empty() ? 1 : s.children.size();
            const int32_t first = (int32_t)s_body.size();
            any_children = any_children || !s.children.empty();
            for (size_t c = 0; c < nc; ++c) {
                const std::vector<float>& v = s.children.empty() ? s.verts : s.children[c];
                proxy_body_.push_back(gpu_body_[i]);
                proxy_shape_.push_back(sid);
                proxy_child_.push_back((uint32_t)c);
                s_body.push_back(i);
                s_kind.push_back(s.kind);
                s_owner.push_back(s.children.empty() ? -1 : first);
                s_voff.push_back((uint32_t)(verts.size() / 2));
                s_nv.push_back((uint32_t)(v.size() / 2));
                verts.insert(verts.end(), v.begin(), v.end());
                s_radius.push_back(s.radius);
                s_density.push_back(s.density);
                s_friction.push_back(s.friction);
                s_restitution.push_back(s.restitution);
                s_filter.insert(s_filter.end(), {s.category, s.mask, s.group, s.sensor});
            }
        }
    }
    const uint32_t S = (uint32_t)s_body.size();
    std::vector<uint32_t> j_bodies;
    std::vector<float> j_anchor, j_param, j_extra;
    std::vector<int32_t> j_flags, j_type;
    // a gear names its coupled joints by ID; the batch takes their batch indices
    std::vector<uint32_t> joint_gpu(joints_.size(), ~0u);
    for (uint32_t j = 0, k = 0; j < joints_.size(); ++j)
        if (joint_live_[j]) joint_gpu[j] = k++;
    for (uint32_t j = 0; j < joints_.size(); ++j) {
        if (!joint_live_[j]) continue;
        HostJoint x = joints_[j];
        if (x.kind == PRGPU_JOINT_GEAR) {
            for (int k = 0; k < 2; ++k) {
                const auto id = static_cast<uint32_t>(x.extra[k]);
                if (id >= joints_.size() || !joint_live_[id]) throw Error(PRGPU_EINVAL, "gear joint: coupled joint destroyed");
                x.extra[k] = static_cast<float>(joint_gpu[id]);
            }
        }
        j_bodies.insert(j_bodies.end(), {body_gpu_[x.body_a], body_gpu_[x.body_b]});
        j_anchor.insert(j_anchor.end(), {x.anchor_a[0], x.anchor_a[1], x.anchor_b[0], x.anchor_b[1]});
        j_param.insert(j_param.end(), {x.reference_angle, x.lower, x.upper, x.motor_speed, x.max_motor_torque, 0.f});
        j_flags.insert(j_flags.end(), {x.enable_limit, x.enable_motor, x.collide_connected});
        j_type.push_back(x.kind);
        j_extra.insert(j_extra.end(), x.extra, x.extra + 8);
    }
    const uint32_t J = (uint32_t)j_bodies.size() / 2;
    prgpu_batch_desc d{};
    d.n_worlds = 1;
    d.world_body_count = &N; d.world_shape_count = &S; d.world_joint_count = &J;
    d.n_bodies = N; d.body_type = type.data(); d.body_pos = pos.data(); d.body_vel = vel.data();
    d.body_acc = acc.data(); d.body_damp = damp.data(); d.body_flags = flags.data();
    d.n_shapes = S; d.shape_body = s_body.data(); d.shape_kind = s_kind.data(); d.shape_voff = s_voff.data();
    d.shape_nv = s_nv.data(); d.shape_radius = s_radius.data(); d.shape_density = s_density.data();
    d.shape_friction = s_friction.data(); d.shape_restitution = s_restitution.data(); d.shape_filter = s_filter.data();
    d.n_verts = (uint32_t)(verts.size() / 2); d.verts = verts.data();
    d.n_joints = J; d.joint_bodies = j_bodies.data(); d.joint_anchors = j_anchor.data(); d.joint_params = j_param.data();
    d.joint_flags = j_flags.data(); d.joint_type = j_type.data(); d.joint_extra = j_extra.data();
    d.shape_owner = any_children ? s_owner.data() : nullptr;
    std::vector<float> mass4;
    if (any_mass) {
        // mass data from the shapes, then the bodies that set their own
        mass4.assign(4 * (size_t)N, 0.f);
        Check(prgpu_prepare_bodies(&d, nullptr, nullptr, mass4.data()), "mass data");
        for (uint32_t i = 0; i < N; ++i) {
            const HostBody& b = bodies_[gpu_body_[i]];
            if (!b.explicit_mass || b.type != PRGPU_DYNAMIC) continue;
            mass4[4 * i] = b.inv_mass; mass4[4 * i + 1] = b.inv_rot_inertia;
            mass4[4 * i + 2] = b.lcx; mass4[4 * i + 3] = b.lcy;
        }
        d.body_mass = mass4.data();
    }
    Check(prgpu_world_create(&d, device_, &gpu_), "prgpu_world_create");
    rebuild_ = false;
    // the reference's contact containers grow without bound: so do the batch's
    Check(prgpu_set_capacity_growth(gpu_, 1), "prgpu_set_capacity_growth");
    if (solve_records_) Check(prgpu_set_solve_records(gpu_, 1), "prgpu_set_solve_records");
    if (sub_stepping_) Check(prgpu_set_sub_stepping(gpu_, 1), "prgpu_set_sub_stepping");
    state_dirty_.assign(bodies_.size(), false);
    lc_.assign(2 * (size_t)N, 0.f);
    std::vector<float> m(4 * (size_t)N), p(3 * (size_t)N);
    Check(prgpu_download_bodies(gpu_, p.data(), nullptr, nullptr, m.data(), nullptr, nullptr), "download");
    for (uint32_t i = 0; i < N; ++i) {
        lc_[2 * i] = m[4 * i + 2]; lc_[2 * i + 1] = m[4 * i + 3];
        HostBody& b = bodies_[gpu_body_[i]];
        b.inv_mass = m[4 * i]; b.inv_rot_inertia = m[4 * i + 1]; b.lcx = m[4 * i + 2]; b.lcy = m[4 * i + 3];
        b.cx = p[3 * i]; b.cy = p[3 * i + 1];
    }
}

void HostWorld::UploadStates() {
    for (uint32_t id = 0; id < state_dirty_.size(); ++id) {
        if (!state_dirty_[id] || !body_live_[id]) continue;
        const uint32_t i = body_gpu_[id];
        const HostBody& b = bodies_[id];
        // the ABI takes the centre of mass: origin + R(angle) local centre
        const float c = std::cos(b.angle), s = std::sin(b.angle);
        const float lx = lc_[2 * i], ly = lc_[2 * i + 1];
        const float p3[3] = {b.x + (c * lx - s * ly), b.y + (s * lx + c * ly), b.angle};
        const float v3[3] = {b.vx, b.vy, b.w};
        Check(prgpu_upload_body_states(gpu_, i, 1, p3, v3), "prgpu_upload_body_states");
        state_dirty_[id] = false;
    }
}

void HostWorld::Pull() {
    const uint32_t N = (uint32_t)gpu_body_.size();
    std::vector<float> p(3 * (size_t)N), v(3 * (size_t)N), xf(4 * (size_t)N), uat(N);
    std::vector<uint32_t> fl(N);
    Check(prgpu_download_bodies(gpu_, p.data(), v.data(), xf.data(), nullptr, uat.data(), fl.data()), "download");
    for (uint32_t i = 0; i < N; ++i) {
        HostBody& b = bodies_[gpu_body_[i]];
        b.x = xf[4 * i]; b.y = xf[4 * i + 1]; b.angle = p[3 * i + 2];
        b.cx = p[3 * i]; b.cy = p[3 * i + 1];
        b.vx = v[3 * i]; b.vy = v[3 * i + 1]; b.w = v[3 * i + 2];
        b.under_active_time = uat[i];
        if (fl[i] & 1u) b.flags |= PRGPU_BODY_AWAKE; else b.flags &= ~(uint32_t)PRGPU_BODY_AWAKE;
    }
}

prgpu_step_stats HostWorld::Step(const prgpu_step_conf& conf) {
    prgpu_step_stats st{};
    if (rebuild_) {
        Drop();
        bool any = false;
        for (bool l : body_live_) any = any || l;
        if (!any) return st;  // an empty world steps trivially
        Build();
    } else {
        UploadStates();
    }
    Check(prgpu_step(gpu_, &conf, &st), "prgpu_step");
    Pull();
    contacts_valid_ = false;
    return st;
}

const std::vector<HostContact>& HostWorld::Contacts() {
    if (contacts_valid_) return contacts_;
    contacts_.clear();
    if (!gpu_) return contacts_;
    uint32_t nc = 0;
    Check(prgpu_get_counts(gpu_, nullptr, nullptr, nullptr, nullptr, &nc), "counts");
    std::vector<uint32_t> pr(2 * (size_t)nc + 2), bd(2 * (size_t)nc + 2), fl(nc + 1), ft(2 * (size_t)nc + 2);
    std::vector<int32_t> meta(2 * (size_t)nc + 2);
    std::vector<float> head(4 * (size_t)nc + 4), pts(8 * (size_t)nc + 8);
    uint32_t n = 0;
    Check(prgpu_download_contacts(gpu_, nc, &n, pr.data(), bd.data(), fl.data(), meta.data(), head.data(), pts.data(),
                                  ft.data()), "prgpu_download_contacts");
    std::vector<uint32_t> slots(n + 1);
    std::vector<float> mat(4 * (size_t)n + 4);
    std::vector<uint64_t> seq(n + 1);
    uint32_t n2 = 0, n3 = 0;
    Check(prgpu_download_contact_state(gpu_, n, &n2, slots.data(), mat.data()), "prgpu_download_contact_state");
    Check(prgpu_download_contact_seq(gpu_, n, &n3, seq.data()), "prgpu_download_contact_seq");
    if (n2 != n || n3 != n) throw Error(PRGPU_ESTATE, "contact downloads disagree");
    contacts_.resize(n);
    for (uint32_t k = 0; k < n; ++k) {
        HostContact& c = contacts_[k];
        c.slot = slots[k];
        c.seq = seq[k];
        c.friction = mat[4 * k]; c.restitution = mat[4 * k + 1]; c.tangent_speed = mat[4 * k + 2];
        c.enabled = mat[4 * k + 3] != 0.f;
        c.proxy_a = leaf_id(pr[2 * k]); c.proxy_b = leaf_id(pr[2 * k + 1]);
        c.body_a = proxy_body_[pr[2 * k]]; c.shape_a = proxy_shape_[pr[2 * k]]; c.child_a = proxy_child_[pr[2 * k]];
        c.body_b = proxy_body_[pr[2 * k + 1]]; c.shape_b = proxy_shape_[pr[2 * k + 1]];
        c.child_b = proxy_child_[pr[2 * k + 1]];
        c.touching = (fl[k] & 1u) != 0u; c.sensor = (fl[k] & 2u) != 0u;
        c.type = meta[2 * k]; c.count = meta[2 * k + 1];
        c.local_normal[0] = head[4 * k]; c.local_normal[1] = head[4 * k + 1];
        c.local_point[0] = head[4 * k + 2]; c.local_point[1] = head[4 * k + 3];
        for (int j = 0; j < 2; ++j) {
            c.point[j][0] = pts[8 * k + 4 * j]; c.point[j][1] = pts[8 * k + 4 * j + 1];
            c.normal_impulse[j] = pts[8 * k + 4 * j + 2]; c.tangent_impulse[j] = pts[8 * k + 4 * j + 3];
            c.feature[j] = ft[2 * k + j];
        }
    }
    contacts_valid_ = true;
    return contacts_;
}

void HostWorld::SetSubStepping(bool enabled) {
    sub_stepping_ = enabled;
    if (gpu_) Check(prgpu_set_sub_stepping(gpu_, enabled ? 1 : 0), "prgpu_set_sub_stepping");
}

bool HostWorld::StepComplete() {
    if (!gpu_) return true;
    int complete = 1;
    Check(prgpu_get_step_complete(gpu_, 0, &complete), "prgpu_get_step_complete");
    return complete != 0;
}

void HostWorld::SetSolveRecords(bool enabled) {
    if (enabled == solve_records_) return;
    solve_records_ = enabled;
    if (gpu_) Check(prgpu_set_solve_records(gpu_, enabled ? 1 : 0), "prgpu_set_solve_records");
}

std::vector<HostSolveRecord> HostWorld::SolveRecords() {
    std::vector<HostSolveRecord> out;
    if (!gpu_) return out;
    uint32_t n = 0;
    Check(prgpu_download_solve_records(gpu_, 0, &n, nullptr, nullptr, nullptr), "prgpu_download_solve_records");
    if (n == 0) return out;
    std::vector<uint32_t> slots(n), info(n);
    std::vector<float> imp(4 * (size_t)n);
    uint32_t m = 0;
    Check(prgpu_download_solve_records(gpu_, n, &m, slots.data(), info.data(), imp.data()),
          "prgpu_download_solve_records");
    out.resize(m);
    for (uint32_t k = 0; k < m; ++k) {
        HostSolveRecord& r = out[k];
        r.slot = slots[k];
        r.phases = info[k] & 7u;
        r.solved = (info[k] & 8u) != 0u;
        r.count = (int32_t)((info[k] >> 4) & 15u);
        r.iter = (info[k] >> 8) & 255u;
        for (int j = 0; j < 2; ++j) {
            r.normal_impulse[j] = imp[4 * k + 2 * j];
            r.tangent_impulse[j] = imp[4 * k + 2 * j + 1];
        }
    }
    return out;
}

void HostWorld::SetContact(uint32_t slot, bool enabled, float friction, float restitution, float tangent_speed) {
    if (!gpu_ || rebuild_) throw Error(PRGPU_EINVAL, "no such contact");
    Check(prgpu_set_contact(gpu_, slot, enabled ? 1 : 0, friction, restitution, tangent_speed), "prgpu_set_contact");
    contacts_valid_ = false;
}

void HostWorld::SetManifold(uint32_t slot, int32_t type, int32_t count, const float head4[4], const float pts8[8]) {
    if (!gpu_ || rebuild_) throw Error(PRGPU_EINVAL, "no such contact");
    Check(prgpu_set_manifold(gpu_, slot, type, count, head4, pts8), "prgpu_set_manifold");
    contacts_valid_ = false;
}

void HostWorld::Proxies(std::vector<float>& aabb4, std::vector<uint32_t>& body_shape_child3) {
    aabb4.clear();
    body_shape_child3.clear();
    if (!gpu_) return;
    aabb4.resize(4 * proxy_body_.size());
    Check(prgpu_download_proxies(gpu_, aabb4.data()), "prgpu_download_proxies");
    for (size_t k = 0; k < proxy_body_.size(); ++k)
        body_shape_child3.insert(body_shape_child3.end(), {proxy_body_[k], proxy_shape_[k], proxy_child_[k]});
}

uint32_t HostWorld::ProxyOf(uint32_t shape, uint32_t child) const {
    for (size_t k = 0; k < proxy_shape_.size(); ++k)
        if (proxy_shape_[k] == shape && proxy_child_[k] == child) return (uint32_t)k;
    return ~0u;
}

}  // namespace prgpu
