// pm_scene.cpp -- seeded synthetic multi-view scenes (see pm_scene.h).
//
// Geometry: infinite slanted planes plus oriented boxes. Rendering: one ray per pixel
// centre; boxes are binned into 16x16-pixel screen tiles by their projected corners so
// large box counts stay cheap. All arithmetic is double precision; the build uses
// -ffp-contract=off so x86_64 and aarch64 render the same images.
#include "pm_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct Vec3 {
    double x, y, z;
};
inline Vec3 operator+(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 operator-(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 operator*(double s, Vec3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(Vec3 a, Vec3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline Vec3 normalize(Vec3 a) { return (1.0 / std::sqrt(dot(a, a))) * a; }

// splitmix64: the scene's own deterministic stream.
struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * uniform(); }
};

inline uint32_t hash32(uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    uint64_t h = 0x243F6A8885A308D3ull;
    uint32_t in[4] = {a, b, c, d};
    for (uint32_t v : in) {
        h ^= v;
        h *= 0x100000001B3ull;
        h ^= h >> 29;
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 32;
    }
    return (uint32_t)h;
}

// Value noise: hashed lattice values, C1 (smoothstep) interpolation, three octaves.
inline double lattice(uint32_t id, uint32_t octave, int64_t ix, int64_t iy)
{
    return (double)(hash32(id, octave, (uint32_t)ix, (uint32_t)iy) >> 8) * (1.0 / 16777216.0);
}

double value_noise(uint32_t id, double u, double v)
{
    double total = 0.0, amp = 1.0, norm = 0.0, freq = 1.0;
    for (uint32_t o = 0; o < 3; ++o) {
        double su = u * freq, sv = v * freq;
        double fu = std::floor(su), fv = std::floor(sv);
        int64_t iu = (int64_t)fu, iv = (int64_t)fv;
        double au = su - fu, av = sv - fv;
        au = au * au * (3.0 - 2.0 * au);
        av = av * av * (3.0 - 2.0 * av);
        double v00 = lattice(id, o, iu, iv), v10 = lattice(id, o, iu + 1, iv);
        double v01 = lattice(id, o, iu, iv + 1), v11 = lattice(id, o, iu + 1, iv + 1);
        double top = v00 + au * (v10 - v00), bot = v01 + au * (v11 - v01);
        total += amp * (top + av * (bot - top));
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return total / norm;
}

struct Plane {
    Vec3 n;       // unit normal, facing the cameras (n.z < 0)
    double d;     // n . X = d on the plane
    Vec3 e1, e2;  // in-plane basis for texture coordinates
    Vec3 origin;
    double cell;  // texture cell size (world units)
    double mean, contrast;
    uint32_t id;
};

struct Box {
    Vec3 c;        // centre
    Vec3 ax[3];    // local axes (rows of the rotation)
    double h[3];   // half extents
    double cell;
    double mean, contrast;
    uint32_t id;
};

}  // namespace

struct pm_scene {
    std::vector<Plane> planes;
    std::vector<Box> boxes;
    double z_pivot;
};

namespace {

Vec3 random_unit(Rng &rng)
{
    for (;;) {
        Vec3 v{rng.range(-1, 1), rng.range(-1, 1), rng.range(-1, 1)};
        double l = dot(v, v);
        if (l > 1e-4 && l <= 1.0) return normalize(v);
    }
}

void basis_for(Vec3 n, Vec3 &e1, Vec3 &e2)
{
    Vec3 a = std::fabs(n.x) < 0.9 ? Vec3{1, 0, 0} : Vec3{0, 1, 0};
    e1 = normalize(cross(a, n));
    e2 = cross(n, e1);
}

// Nearest hit along origin + s * dir (s > 0). Returns s, or -1 when nothing is hit.
struct Hit {
    double s;
    double shade;
};

inline double surface_value(uint32_t id, double u, double v, double cell, double mean,
                            double contrast)
{
    double nv = value_noise(id, u / cell, v / cell);
    double val = mean + contrast * (2.0 * nv - 1.0);
    return val < 0.0 ? 0.0 : (val > 255.0 ? 255.0 : val);
}

inline void hit_plane(const Plane &p, Vec3 o, Vec3 dir, Hit &best)
{
    double den = dot(p.n, dir);
    if (std::fabs(den) < 1e-12) return;
    double s = (p.d - dot(p.n, o)) / den;
    if (!(s > 1e-9) || s >= best.s) return;
    Vec3 x = o + s * dir - p.origin;
    best.s = s;
    best.shade = surface_value(p.id, dot(x, p.e1), dot(x, p.e2), p.cell, p.mean, p.contrast);
}

inline void hit_box(const Box &b, Vec3 o, Vec3 dir, Hit &best)
{
    Vec3 rel = o - b.c;
    double lo[3], ld[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = dot(b.ax[k], rel);
        ld[k] = dot(b.ax[k], dir);
    }
    double t0 = -1e300, t1 = 1e300;
    int face = -1;
    for (int k = 0; k < 3; ++k) {
        if (std::fabs(ld[k]) < 1e-15) {
            if (lo[k] < -b.h[k] || lo[k] > b.h[k]) return;
            continue;
        }
        double inv = 1.0 / ld[k];
        double ta = (-b.h[k] - lo[k]) * inv, tb = (b.h[k] - lo[k]) * inv;
        if (ta > tb) std::swap(ta, tb);
        if (ta > t0) { t0 = ta; face = k; }
        if (tb < t1) t1 = tb;
        if (t0 > t1) return;
    }
    if (face < 0 || !(t0 > 1e-9) || t0 >= best.s) return;
    double q[3];
    for (int k = 0; k < 3; ++k) q[k] = lo[k] + t0 * ld[k];
    int a = (face + 1) % 3, c = (face + 2) % 3;
    uint32_t fid = b.id * 8u + (uint32_t)face * 2u + (q[face] > 0 ? 1u : 0u);
    best.s = t0;
    best.shade = surface_value(fid, q[a], q[c], b.cell, b.mean, b.contrast);
}

}  // namespace

extern "C" pm_scene *pm_scene_create(uint64_t seed, int n_planes, int n_boxes, double depth_near,
                                     double depth_far, int width, int height, double focal)
{
    if (n_planes < 1 || n_boxes < 0 || !(depth_near > 0) || !(depth_far > depth_near) ||
        width < 8 || height < 8 || !(focal > 0))
        return nullptr;
    pm_scene *sc = new pm_scene();
    Rng rng{seed * 0x9E3779B97F4A7C15ull + 0x1234567ull};
    const double span = depth_far - depth_near;
    sc->z_pivot = depth_near + 0.5 * span;
    const double half_fov_x = 0.5 * width / focal, half_fov_y = 0.5 * height / focal;
    const double max_tilt = n_boxes > 0 ? 35.0 : 25.0;
    const double tan_max = std::tan(max_tilt * M_PI / 180.0);

    // Planes: the envelope stays inside the range at every ref-view pixel.
    for (int i = 0; i < n_planes; ++i) {
        Plane p{};
        for (int attempt = 0;; ++attempt) {
            double zc = n_boxes > 0 ? rng.range(depth_near + 0.35 * span, depth_far - 0.08 * span)
                                    : rng.range(depth_near + 0.28 * span, depth_far - 0.25 * span);
            double tilt = std::atan(tan_max * std::sqrt(rng.uniform()));
            double az = rng.range(0, 2 * M_PI);
            Vec3 n{std::sin(tilt) * std::cos(az), std::sin(tilt) * std::sin(az), -std::cos(tilt)};
            // Depth of the plane along ray (rx, ry, 1): z = (n . P) / (n . r).
            double np = n.z * zc;
            double zmin = 1e300, zmax = -1e300;
            for (int cx = -1; cx <= 1; cx += 2)
                for (int cy = -1; cy <= 1; cy += 2) {
                    double nr = n.x * cx * half_fov_x + n.y * cy * half_fov_y + n.z;
                    double z = np / nr;
                    if (!(z > 0)) { zmin = -1; break; }
                    zmin = std::min(zmin, z);
                    zmax = std::max(zmax, z);
                }
            if ((zmin >= depth_near + 0.05 * span && zmax <= depth_far - 0.03 * span) ||
                attempt > 200) {
                p.n = n;
                p.origin = Vec3{0, 0, zc};
                p.d = dot(n, p.origin);
                break;
            }
        }
        basis_for(p.n, p.e1, p.e2);
        double px_world = sc->z_pivot / focal;
        p.cell = rng.range(4.0, 7.0) * px_world;
        p.mean = rng.range(90, 165);
        p.contrast = rng.range(55, 85);
        p.id = 0x100u + (uint32_t)i;
        sc->planes.push_back(p);
    }

    // Boxes inside the ref frustum, in front of the plane envelope.
    for (int i = 0; i < n_boxes; ++i) {
        Box b{};
        double z = rng.range(depth_near + 0.08 * span, depth_near + 0.62 * span);
        double xf = rng.range(-0.9, 0.9) * half_fov_x, yf = rng.range(-0.9, 0.9) * half_fov_y;
        b.c = Vec3{xf * z, yf * z, z};
        double size = z * rng.range(0.015, 0.05);
        for (int k = 0; k < 3; ++k) b.h[k] = size * rng.range(0.5, 1.5);
        // random rotation from a random axis and angle (Rodrigues)
        Vec3 axis = random_unit(rng);
        double ang = rng.range(0, M_PI);
        double c = std::cos(ang), s = std::sin(ang), C = 1 - c;
        double R[9] = {c + axis.x * axis.x * C, axis.x * axis.y * C - axis.z * s,
                       axis.x * axis.z * C + axis.y * s, axis.y * axis.x * C + axis.z * s,
                       c + axis.y * axis.y * C, axis.y * axis.z * C - axis.x * s,
                       axis.z * axis.x * C - axis.y * s, axis.z * axis.y * C + axis.x * s,
                       c + axis.z * axis.z * C};
        for (int k = 0; k < 3; ++k) b.ax[k] = Vec3{R[3 * k], R[3 * k + 1], R[3 * k + 2]};
        b.cell = rng.range(4.0, 7.0) * z / focal;
        b.mean = rng.range(70, 185);
        b.contrast = rng.range(50, 80);
        b.id = 0x10000u + (uint32_t)i;
        sc->boxes.push_back(b);
    }
    return sc;
}

extern "C" void pm_scene_destroy(pm_scene *scene) { delete scene; }

extern "C" double pm_scene_pivot_depth(const pm_scene *scene) { return scene->z_pivot; }

extern "C" void pm_scene_camera(const pm_scene *scene, double yaw_deg, double pitch_deg,
                                int width, int height, double focal, double K[9], double R[9],
                                double t[3])
{
    const double th = yaw_deg * M_PI / 180.0, ph = pitch_deg * M_PI / 180.0;
    Vec3 f{std::sin(th) * std::cos(ph), std::sin(ph), std::cos(th) * std::cos(ph)};
    Vec3 xa = normalize(Vec3{std::cos(th), 0, -std::sin(th)});
    Vec3 ya = cross(f, xa);
    Vec3 pivot{0, 0, scene->z_pivot};
    Vec3 C = pivot - scene->z_pivot * f;
    R[0] = xa.x; R[1] = xa.y; R[2] = xa.z;
    R[3] = ya.x; R[4] = ya.y; R[5] = ya.z;
    R[6] = f.x;  R[7] = f.y;  R[8] = f.z;
    for (int i = 0; i < 3; ++i) t[i] = -(R[3 * i] * C.x + R[3 * i + 1] * C.y + R[3 * i + 2] * C.z);
    K[0] = focal; K[1] = 0; K[2] = 0.5 * width;
    K[3] = 0; K[4] = focal; K[5] = 0.5 * height;
    K[6] = 0; K[7] = 0; K[8] = 1;
}

extern "C" int pm_scene_render(const pm_scene *scene, const double K[9], const double R[9],
                               const double t[3], int width, int height, uint8_t *image,
                               float *depth)
{
    const double fx = K[0], skew = K[1], cx = K[2], fy = K[4], cy = K[5];
    // camera centre C = -R^T t
    Vec3 C{-(R[0] * t[0] + R[3] * t[1] + R[6] * t[2]), -(R[1] * t[0] + R[4] * t[1] + R[7] * t[2]),
           -(R[2] * t[0] + R[5] * t[1] + R[8] * t[2])};
    // Bin boxes into 16x16 screen tiles by their projected corners.
    const int tile = 16, tw = (width + tile - 1) / tile, th = (height + tile - 1) / tile;
    std::vector<std::vector<int>> bins((size_t)tw * th);
    for (size_t bi = 0; bi < scene->boxes.size(); ++bi) {
        const Box &b = scene->boxes[bi];
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        bool behind = false;
        for (int corner = 0; corner < 8; ++corner) {
            Vec3 X = b.c;
            for (int k = 0; k < 3; ++k) X = X + ((corner >> k) & 1 ? b.h[k] : -b.h[k]) * b.ax[k];
            double xc = R[0] * X.x + R[1] * X.y + R[2] * X.z + t[0];
            double yc = R[3] * X.x + R[4] * X.y + R[5] * X.z + t[1];
            double zc = R[6] * X.x + R[7] * X.y + R[8] * X.z + t[2];
            if (!(zc > 1e-6)) { behind = true; break; }
            double u = (fx * xc + skew * yc) / zc + cx, v = fy * yc / zc + cy;
            xmin = std::min(xmin, u); xmax = std::max(xmax, u);
            ymin = std::min(ymin, v); ymax = std::max(ymax, v);
        }
        int tx0 = 0, tx1 = tw - 1, ty0 = 0, ty1 = th - 1;
        if (!behind) {
            if (xmax < 0 || ymax < 0 || xmin > width || ymin > height) continue;
            tx0 = std::max(0, (int)std::floor(xmin) / tile - 1);
            tx1 = std::min(tw - 1, (int)std::floor(std::min(xmax, (double)width)) / tile + 1);
            ty0 = std::max(0, (int)std::floor(ymin) / tile - 1);
            ty1 = std::min(th - 1, (int)std::floor(std::min(ymax, (double)height)) / tile + 1);
        }
        for (int ty = ty0; ty <= ty1; ++ty)
            for (int tx = tx0; tx <= tx1; ++tx) bins[(size_t)ty * tw + tx].push_back((int)bi);
    }
    int misses = 0;
    #pragma omp parallel for schedule(dynamic, 4) reduction(+ : misses)
    for (int y = 0; y < height; ++y) {
        for (int x = 0; x < width; ++x) {
            // ray direction in camera coordinates with z = 1, then in world coordinates
            double yn = (y + 0.5 - cy) / fy;
            double xn = (x + 0.5 - cx - skew * yn) / fx;
            Vec3 dir{R[0] * xn + R[3] * yn + R[6], R[1] * xn + R[4] * yn + R[7],
                     R[2] * xn + R[5] * yn + R[8]};
            Hit best{1e300, 0.0};
            for (const Plane &p : scene->planes) hit_plane(p, C, dir, best);
            const std::vector<int> &bin = bins[(size_t)(y / tile) * tw + x / tile];
            for (int bi : bin) hit_box(scene->boxes[(size_t)bi], C, dir, best);
            size_t o = (size_t)y * width + x;
            if (best.s >= 1e299) {
                ++misses;
                image[o] = 0;
                if (depth) depth[o] = 0.0f;
            } else {
                image[o] = (uint8_t)std::floor(best.shade + 0.5);
                if (depth) depth[o] = (float)best.s;  // z-depth: the ray has camera z = 1
            }
        }
    }
    return misses;
}
