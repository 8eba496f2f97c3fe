// Foam cluster dynamics restated from the reference's CPU code, with its O(n^2) loops as
// written: FoamSimulator::compute_forces / compute_buoyancy / compute_interaction_force /
// compute_drag / step / handle_coalescence (foam_dynamics.rs:62-238) and
// BubbleCluster::update_connections / merge_bubbles / remove_bubble (foam.rs:262-405),
// BubbleConnection::new (foam.rs:107-141). TEST INFRASTRUCTURE (see oracle.h).
//
// The arithmetic of the third-party vector type, glam 0.29.3 (Cargo.lock:1071-1072), restated:
// Vec3 is plain f32 x, y, z with component-wise operators; length() = sqrt(x*x + y*y + z*z)
// summed left to right; v / s divides each component; dot sums left to right;
// normalize_or_zero() multiplies by 1 / length() when that is finite and > 0, else gives zero.
// f32::powi(2) and powi(3) are x*x and x*(x*x) (the compiler's expansion of powi). The
// reference's powf(x, 1.5) (Hertz contact) and powf(x, 1/3) (merged radius) go to libm. Here
// x^1.5 is the library's own evaluation (the same operations as the CUDA kernel): the correctly
// rounded sqrt s, the product p = x s, and the exact FMA residuals of the product (x s - p) and of
// the root (x - s^2, times s / 2), added once; this is the correctly rounded x^1.5 but for
// near-ties (about one argument in 10^6). x^(1/3) is rounded once from double, as the kernel does.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

constexpr float kPi = 3.14159265358979323846f;

struct V3 {
    float x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize_or_zero(V3 a) {
    const float rcp = 1.0f / length(a);
    if (std::isfinite(rcp) && rcp > 0.0f) return a * rcp;
    return {0.0f, 0.0f, 0.0f};
}

// x^1.5 for x > 0 (the Hertz contact term, foam_dynamics.rs:144)
inline float pow15(float x) {
    const float s = std::sqrt(x);
    const float p = x * s;
    const float e = std::fma(x, s, -p);
    const float r = std::fma(-s, s, x);
    const float c = std::fma(0.5f * r, s, e);
    return p + c;
}

struct Bubble {
    uint32_t id;
    V3 position;
    float radius;
    V3 velocity;
    float thickness_nm;
};

inline float volume(const Bubble &b) { return (4.0f / 3.0f) * kPi * (b.radius * (b.radius * b.radius)); }

struct Sim {
    const sbs_foam_physics &p;
    V3 gravity;
};

// compute_buoyancy (foam_dynamics.rs:99-113)
V3 buoyancy(const Sim &s, const Bubble &b) {
    const float shell_volume = 4.0f * kPi * (b.radius * b.radius) * (b.thickness_nm * 1e-9f);
    const float film_mass = shell_volume * s.p.density;
    const float air_density = 1.2f;
    const float buoyancy_force = volume(b) * air_density * length(s.gravity);
    const float net = film_mass * length(s.gravity) - buoyancy_force;
    return normalize_or_zero(s.gravity) * std::fmax(net, 0.0f);
}

// compute_interaction_force (foam_dynamics.rs:118-160): the force on a; b receives its negation
V3 interaction(const Sim &s, const Bubble &a, const Bubble &b) {
    const V3 delta = b.position - a.position;
    const float distance = length(delta);
    if (distance < 1e-6f) return {0.0f, 0.0f, 0.0f};
    const V3 direction = delta / distance;
    const float sum_radii = a.radius + b.radius;
    V3 force{0.0f, 0.0f, 0.0f};
    if (distance < sum_radii * 3.0f && distance > sum_radii) {
        const float vdw = s.p.van_der_waals_strength * a.radius * b.radius / (distance * distance);
        force = force + direction * vdw;
    }
    const float overlap = sum_radii - distance;
    if (overlap > 0.0f) {
        const float repulsion = s.p.repulsion_stiffness * pow15(overlap);
        force = force - direction * repulsion;
    }
    const float contact_threshold = sum_radii * 1.2f;
    const float min_distance = sum_radii * 0.95f;
    if (distance < contact_threshold && distance > min_distance) {
        const float adhesion = 2.0f * (contact_threshold - distance);
        force = force + direction * adhesion;
    }
    return force;
}

// compute_drag (foam_dynamics.rs:163-167)
V3 drag(const Sim &s, const Bubble &b) {
    const float drag_coeff = 6.0f * kPi * s.p.viscosity * b.radius;
    return -b.velocity * drag_coeff;
}

// compute_forces (foam_dynamics.rs:62-94): the all-pairs loop in its own accumulation order
void forces(const Sim &s, const std::vector<Bubble> &bs, std::vector<V3> &f) {
    const size_t n = bs.size();
    f.assign(n, V3{0.0f, 0.0f, 0.0f});
    for (size_t i = 0; i < n; ++i) {
        f[i] = f[i] + buoyancy(s, bs[i]);
        for (size_t j = i + 1; j < n; ++j) {
            const V3 fij = interaction(s, bs[i], bs[j]);
            f[i] = f[i] + fij;
            f[j] = f[j] + (-fij);
        }
        f[i] = f[i] + drag(s, bs[i]);
    }
}

// BubbleConnection::new (foam.rs:107-141)
sbs_bubble_connection connection(const Bubble &a, const Bubble &b, float surface_tension) {
    const V3 delta = b.position - a.position;
    const float distance = length(delta);
    const V3 normal = delta / distance;
    const float t = a.radius / (a.radius + b.radius);
    const V3 contact = a.position + delta * t;
    const float p_a = 4.0f * surface_tension / a.radius;
    const float p_b = 4.0f * surface_tension / b.radius;
    const float delta_p = p_a - p_b;
    sbs_bubble_connection c;
    c.bubble_a = a.id;
    c.bubble_b = b.id;
    c.contact_point[0] = contact.x;
    c.contact_point[1] = contact.y;
    c.contact_point[2] = contact.z;
    c.contact_normal[0] = normal.x;
    c.contact_normal[1] = normal.y;
    c.contact_normal[2] = normal.z;
    c.wall_curvature_radius = std::fabs(delta_p) > 1e-6f ? 2.0f * surface_tension / delta_p : INFINITY;
    c.wall_thickness_nm = (a.thickness_nm + b.thickness_nm) / 2.0f * 0.8f;
    return c;
}

// update_connections (foam.rs:322-364): every pair i < j in contact or within 30 % of r_i
void update_connections(const Sim &s, const std::vector<Bubble> &bs, std::vector<sbs_bubble_connection> &out) {
    out.clear();
    const size_t n = bs.size();
    for (size_t i = 0; i < n; ++i)
        for (size_t j = i + 1; j < n; ++j) {
            const Bubble &a = bs[i], &b = bs[j];
            const float overlap = a.radius + b.radius - length(a.position - b.position);
            const float threshold = -a.radius * 0.3f;
            if (overlap > threshold) out.push_back(connection(a, b, s.p.surface_tension));
        }
}

int find(const std::vector<Bubble> &bs, uint32_t id) {
    for (size_t i = 0; i < bs.size(); ++i)
        if (bs[i].id == id) return (int)i;
    return -1;
}

// merge_bubbles (foam.rs:369-405), with remove_bubble (foam.rs:262-272)
void merge(std::vector<Bubble> &bs, std::vector<sbs_bubble_connection> &conns, uint32_t id_a, uint32_t id_b,
           uint32_t &next_id) {
    const int ia = find(bs, id_a), ib = find(bs, id_b);
    if (ia < 0 || ib < 0) return;
    const Bubble a = bs[ia], b = bs[ib];
    const float vol_a = volume(a), vol_b = volume(b);
    const float vol_total = vol_a + vol_b;
    const float base = vol_total * 3.0f / (4.0f * kPi);
    const float new_radius = (float)std::pow((double)base, (double)(1.0f / 3.0f));
    const V3 new_position = (a.position * vol_a + b.position * vol_b) / vol_total;
    const V3 new_velocity = (a.velocity * vol_a + b.velocity * vol_b) / vol_total;
    const float area_a = 4.0f * kPi * (a.radius * a.radius);
    const float area_b = 4.0f * kPi * (b.radius * b.radius);
    const float new_thickness = (a.thickness_nm * area_a + b.thickness_nm * area_b) / (area_a + area_b);
    for (uint32_t id : {id_a, id_b}) {
        const int k = find(bs, id);
        bs.erase(bs.begin() + k);
        std::vector<sbs_bubble_connection> kept;
        for (const auto &c : conns)
            if (c.bubble_a != id && c.bubble_b != id) kept.push_back(c);
        conns.swap(kept);
    }
    Bubble m;
    m.id = next_id++;
    m.position = new_position;
    m.radius = new_radius;
    m.velocity = new_velocity;
    m.thickness_nm = new_thickness;
    bs.push_back(m);
}

std::vector<Bubble> load(uint32_t n, const float *pos, const float *vel, const float *radius, const float *thick,
                         const uint32_t *ids) {
    std::vector<Bubble> bs(n);
    for (uint32_t i = 0; i < n; ++i) {
        bs[i].id = ids ? ids[i] : i;
        bs[i].position = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        bs[i].radius = radius[i];
        bs[i].velocity = vel ? V3{vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]} : V3{0.0f, 0.0f, 0.0f};
        bs[i].thickness_nm = thick ? thick[i] : 500.0f;
    }
    return bs;
}

}  // namespace

extern "C" {

float orc_pow15(float x) { return pow15(x); }

void orc_foam_forces(const sbs_foam_physics *p, uint32_t n, const float *pos, const float *vel, const float *radius,
                     const float *thick, float *out) {
    const Sim s{*p, V3{p->gravity[0], p->gravity[1], p->gravity[2]}};
    const std::vector<Bubble> bs = load(n, pos, vel, radius, thick, nullptr);
    std::vector<V3> f;
    forces(s, bs, f);
    for (uint32_t i = 0; i < n; ++i) {
        out[3 * i] = f[i].x;
        out[3 * i + 1] = f[i].y;
        out[3 * i + 2] = f[i].z;
    }
}

// The forces on the bubbles idx[0..m) alone, in the order compute_forces accumulates them for bubble
// k: -f_jk for j < k ascending (the inner loops of the earlier i), its buoyancy, f_kj for j > k
// ascending, its drag. O(n m): a check of single bubbles in clusters too large for the full loop.
void orc_foam_forces_subset(const sbs_foam_physics *p, uint32_t n, const float *pos, const float *vel,
                            const float *radius, const float *thick, const uint32_t *idx, uint32_t m, float *out) {
    const Sim s{*p, V3{p->gravity[0], p->gravity[1], p->gravity[2]}};
    const std::vector<Bubble> bs = load(n, pos, vel, radius, thick, nullptr);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t q = 0; q < (int64_t)m; ++q) {
        const uint32_t k = idx[q];
        V3 f{0.0f, 0.0f, 0.0f};
        for (uint32_t j = 0; j < k; ++j) f = f + (-interaction(s, bs[j], bs[k]));
        f = f + buoyancy(s, bs[k]);
        for (uint32_t j = k + 1; j < n; ++j) f = f + interaction(s, bs[k], bs[j]);
        f = f + drag(s, bs[k]);
        out[3 * q] = f.x;
        out[3 * q + 1] = f.y;
        out[3 * q + 2] = f.z;
    }
}

uint32_t orc_foam_step(const sbs_foam_physics *p, float dt, uint32_t steps, uint32_t n, float *pos, float *vel,
                       float *radius, float *thick, uint32_t *ids, uint32_t *next_id, sbs_bubble_connection *conn,
                       uint32_t cap, uint32_t *nconn) {
    const Sim s{*p, V3{p->gravity[0], p->gravity[1], p->gravity[2]}};
    std::vector<Bubble> bs = load(n, pos, vel, radius, thick, ids);
    std::vector<V3> f;
    std::vector<sbs_bubble_connection> conns;
    update_connections(s, bs, conns);  // the cluster's connections before any step
    for (uint32_t step = 0; step < steps; ++step) {
        // step (foam_dynamics.rs:172-211)
        forces(s, bs, f);
        for (size_t i = 0; i < bs.size(); ++i) {
            Bubble &b = bs[i];
            const float shell_volume = 4.0f * kPi * (b.radius * b.radius) * (b.thickness_nm * 1e-9f);
            const float mass = std::fmax(shell_volume * p->density, 1e-9f);
            const V3 acceleration = f[i] / mass;
            b.velocity = b.velocity + acceleration * dt;
            b.velocity = b.velocity * p->damping;
            const float max_speed = 0.1f;
            const float speed = length(b.velocity);
            if (speed > max_speed) b.velocity = b.velocity * (max_speed / speed);
            b.position = b.position + b.velocity * dt;
        }
        update_connections(s, bs, conns);
        if (p->coalescence_enabled) {
            // handle_coalescence (foam_dynamics.rs:214-238): the first qualifying connection merges
            for (const auto &c : conns) {
                const int ia = find(bs, c.bubble_a), ib = find(bs, c.bubble_b);
                if (ia < 0 || ib < 0) continue;
                const Bubble &a = bs[ia], &b = bs[ib];
                const V3 normal{c.contact_normal[0], c.contact_normal[1], c.contact_normal[2]};
                const float rel_velocity = dot(b.velocity - a.velocity, normal);
                const float weber = p->density * (rel_velocity * rel_velocity) * a.radius / p->surface_tension;
                if (weber > p->coalescence_threshold) {
                    merge(bs, conns, c.bubble_a, c.bubble_b, *next_id);
                    break;
                }
            }
        }
    }
    const uint32_t m = (uint32_t)bs.size();
    for (uint32_t i = 0; i < m; ++i) {
        pos[3 * i] = bs[i].position.x;
        pos[3 * i + 1] = bs[i].position.y;
        pos[3 * i + 2] = bs[i].position.z;
        vel[3 * i] = bs[i].velocity.x;
        vel[3 * i + 1] = bs[i].velocity.y;
        vel[3 * i + 2] = bs[i].velocity.z;
        radius[i] = bs[i].radius;
        thick[i] = bs[i].thickness_nm;
        ids[i] = bs[i].id;
    }
    *nconn = (uint32_t)conns.size();
    for (uint32_t c = 0; c < conns.size() && c < cap; ++c) conn[c] = conns[c];
    return m;
}

}  // extern "C"
