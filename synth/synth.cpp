// Seeded synthetic RGB-D sequences standing in for the TUM RGB-D recordings
// the reference is run on (MainTum.cc:21-75): analytic scenes rendered to
// uint16 depth (mm), uint8 RGB and uint8 instance masks, with a
// depth-dependent noise model, random dropout and a smooth trajectory.
// Everything is a pure function of (config, frame index): pixels use a
// counter-based hash, so frames can be generated in any order.
#include "sf_synth.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct V3 { double x, y, z; };
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scl(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 unit(V3 a) { return scl(a, 1.0 / std::sqrt(dot(a, a))); }

inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
inline uint64_t key(uint64_t seed, uint64_t a, uint64_t b, uint64_t c) {
  return mix64(seed ^ mix64(a * 0x100000001b3ull ^ mix64(b * 0xc2b2ae3d27d4eb4full ^ mix64(c))));
}
inline double uni(uint64_t k) { return ((k >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
inline double gauss(uint64_t k1, uint64_t k2) {
  double u1 = uni(k1), u2 = uni(k2);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

// Sequential RNG for scene / trajectory layout.
struct Rng {
  uint64_t s;
  double next() { s = mix64(s); return uni(s); }
  double range(double a, double b) { return a + (b - a) * next(); }
};

// 3-D gradient noise (Perlin's construction: quintic fade, hashed lattice
// gradients, trilinear blend of the corner dot products).
double grad_noise(uint64_t seed, double x, double y, double z) {
  double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  long ix = (long)fx, iy = (long)fy, iz = (long)fz;
  double dx = x - fx, dy = y - fy, dz = z - fz;
  auto fade = [](double t) { return t * t * t * (t * (t * 6 - 15) + 10); };
  double u = fade(dx), v = fade(dy), w = fade(dz);
  double acc[2][2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int c = 0; c < 2; ++c) {
        uint64_t h = key(seed, (uint64_t)(ix + a), (uint64_t)(iy + b), (uint64_t)(iz + c));
        double gx = uni(h) * 2 - 1, gy = uni(mix64(h)) * 2 - 1, gz = uni(mix64(h + 1)) * 2 - 1;
        acc[a][b][c] = gx * (dx - a) + gy * (dy - b) + gz * (dz - c);
      }
  auto lerp = [](double a, double b, double t) { return a + (b - a) * t; };
  double x00 = lerp(acc[0][0][0], acc[1][0][0], u), x10 = lerp(acc[0][1][0], acc[1][1][0], u);
  double x01 = lerp(acc[0][0][1], acc[1][0][1], u), x11 = lerp(acc[0][1][1], acc[1][1][1], u);
  return lerp(lerp(x00, x10, v), lerp(x01, x11, v), w);
}

struct Prim {
  int kind;        // 0 sphere, 1 axis-aligned box
  V3 c, h;         // centre; half extents (box) or (r, r, r)
  double rgb[3];   // base colour
  uint8_t cls;     // instance class id for masks (0 = background)
};

}  // namespace

struct sf_synth {
  sf_synth_config cfg;
  V3 lo, hi;               // the enclosing room / corridor (seen from inside)
  std::vector<Prim> prims;
  std::vector<V3> ctrl;    // spline control points
  double room_rgb[3];
};

namespace {

// Ray / scene intersection.  Returns the hit distance along the unit-free
// direction d (camera-frame z = t when d has camera z = 1) and the hit id
// (-1 = enclosure, k = primitive k).
bool intersect(const sf_synth &s, V3 o, V3 d, double &t, int &id) {
  // exit distance from the enclosure box
  double tx = d.x > 0 ? (s.hi.x - o.x) / d.x : (d.x < 0 ? (s.lo.x - o.x) / d.x : 1e30);
  double ty = d.y > 0 ? (s.hi.y - o.y) / d.y : (d.y < 0 ? (s.lo.y - o.y) / d.y : 1e30);
  double tz = d.z > 0 ? (s.hi.z - o.z) / d.z : (d.z < 0 ? (s.lo.z - o.z) / d.z : 1e30);
  t = std::min(tx, std::min(ty, tz));
  id = -1;
  for (size_t k = 0; k < s.prims.size(); ++k) {
    const Prim &p = s.prims[k];
    double th = 1e30;
    if (p.kind == 0) {
      V3 oc = sub(o, p.c);
      double a = dot(d, d), b = 2 * dot(oc, d), c = dot(oc, oc) - p.h.x * p.h.x;
      double disc = b * b - 4 * a * c;
      if (disc >= 0) {
        double sq = std::sqrt(disc);
        double t0 = (-b - sq) / (2 * a);
        if (t0 > 1e-6) th = t0;
      }
    } else {
      double tmin = -1e30, tmax = 1e30;
      const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
      const double cc[3] = {p.c.x, p.c.y, p.c.z}, hh[3] = {p.h.x, p.h.y, p.h.z};
      bool miss = false;
      for (int ax = 0; ax < 3; ++ax) {
        if (std::fabs(dd[ax]) < 1e-12) {
          if (oo[ax] < cc[ax] - hh[ax] || oo[ax] > cc[ax] + hh[ax]) miss = true;
          continue;
        }
        double t1 = (cc[ax] - hh[ax] - oo[ax]) / dd[ax], t2 = (cc[ax] + hh[ax] - oo[ax]) / dd[ax];
        if (t1 > t2) std::swap(t1, t2);
        tmin = std::max(tmin, t1);
        tmax = std::min(tmax, t2);
      }
      if (!miss && tmin <= tmax && tmin > 1e-6) th = tmin;
    }
    if (th < t) { t = th; id = (int)k; }
  }
  return t < 1e29;
}

void build_scene(sf_synth &s) {
  const sf_synth_config &c = s.cfg;
  Rng r{c.seed * 7919 + 17};
  s.room_rgb[0] = 150; s.room_rgb[1] = 140; s.room_rgb[2] = 120;
  if (c.scene == SF_SCENE_CORRIDOR) {
    // 20 m corridor of seeded boxes and pillars.  The world origin lies
    // outside the corridor.
    s.lo = {1.0, -4.5, -1.5};
    s.hi = {21.0, -1.5, 1.5};
    int n = c.n_objects > 0 ? c.n_objects : 24;
    for (int k = 0; k < n; ++k) {
      Prim p;
      bool pillar = (k % 2) == 0;
      double side = (r.next() < 0.5) ? s.lo.y + 0.35 : s.hi.y - 0.35;
      double x = 2.0 + 18.0 * (k + r.next()) / n;
      if (pillar) {
        p.kind = 1;
        p.h = {0.15 + 0.1 * r.next(), 0.15 + 0.1 * r.next(), 1.5};
        p.c = {x, side, 0.0};
      } else {
        p.kind = r.next() < 0.5 ? 1 : 0;
        double rad = r.range(0.2, 0.35);
        p.h = {rad, rad, rad};
        p.c = {x, side, s.lo.z + rad};
      }
      for (int q = 0; q < 3; ++q) p.rgb[q] = r.range(40, 230);
      p.cls = (uint8_t)(1 + (int)(r.next() * 80) % 80);
      s.prims.push_back(p);
    }
  } else {
    // 4 x 4 x 3 m room; centre (3, -3, 0), so the world origin lies outside.
    s.lo = {1.0, -5.0, -1.5};
    s.hi = {5.0, -1.0, 1.5};
    V3 centre = {3.0, -3.0, 0.0};
    int n = c.n_objects > 0 ? c.n_objects : 6;
    for (int k = 0; k < n; ++k) {
      Prim p;
      p.kind = (k % 2 == 0) ? 0 : 1;
      double rad = r.range(0.2, 0.6);
      p.h = {rad, rad, rad};
      if (p.kind == 1) p.h = {rad, r.range(0.2, 0.6), r.range(0.2, 0.6)};
      // keep every surface >= ~0.5 m from the camera path (radius <= 0.6)
      double ang = r.range(0, 6.283185307179586);
      double extent = std::max(p.h.x, std::max(p.h.y, p.h.z)) * 1.42;
      double dist = r.range(1.15 + extent, 2.2);
      p.c = {centre.x + dist * std::cos(ang), centre.y + dist * std::sin(ang), r.range(-1.5 + p.h.z, -0.4)};
      for (int q = 0; q < 3; ++q) p.rgb[q] = r.range(40, 230);
      p.cls = (uint8_t)(1 + (int)(r.next() * 80) % 80);
      s.prims.push_back(p);
    }
    for (int k = 0; k < 8; ++k) {
      double a = r.range(0, 6.283185307179586), rr = r.range(0.0, 0.45);
      s.ctrl.push_back({centre.x + rr * std::cos(a), centre.y + rr * std::sin(a), r.range(-0.25, 0.25)});
    }
  }
}

V3 catmull(const std::vector<V3> &P, double u) {
  int n = (int)P.size();
  int i = (int)std::floor(u);
  double t = u - i;
  auto at = [&](int k) { return P[((k % n) + n) % n]; };
  V3 p0 = at(i - 1), p1 = at(i), p2 = at(i + 1), p3 = at(i + 2);
  double t2 = t * t, t3 = t2 * t;
  auto comp = [&](double a, double b, double c, double d) {
    return 0.5 * ((2 * b) + (-a + c) * t + (2 * a - 5 * b + 4 * c - d) * t2 + (-a + 3 * b - 3 * c + d) * t3);
  };
  return {comp(p0.x, p1.x, p2.x, p3.x), comp(p0.y, p1.y, p2.y, p3.y), comp(p0.z, p1.z, p2.z, p3.z)};
}

// Camera pose (camera -> world; camera x right, y down, z forward).
void pose_at(const sf_synth &s, int i, double T[16]) {
  const sf_synth_config &c = s.cfg;
  V3 pos;
  double yaw, pitch;
  const double deg = 3.141592653589793 / 180.0;
  Rng r{c.seed * 31 + 5};
  double yaw0 = r.range(0, 6.283185307179586);
  if (c.trajectory == SF_TRAJ_CIRCLE) {
    // radius 0.5 m, 2 cm of arc and 1 degree of yaw per frame
    double phi = r.range(0, 6.283185307179586) + i * (0.02 / 0.5);
    pos = {3.0 + 0.5 * std::cos(phi), -3.0 + 0.5 * std::sin(phi), 0.05 * std::sin(i * 0.05)};
    yaw = yaw0 + i * 1.0 * deg;
    pitch = -15.0 * deg + 4.0 * deg * std::sin(i * 0.031);
  } else if (c.trajectory == SF_TRAJ_SPLINE) {
    // ~1.5 cm per frame along a closed Catmull-Rom spline (0.01 of a
    // segment per frame), yaw drifting ~0.8 degree per frame
    pos = catmull(s.ctrl, i * 0.01);
    yaw = yaw0 + i * 0.8 * deg + 10.0 * deg * std::sin(i * 0.013);
    pitch = -15.0 * deg + 6.0 * deg * std::sin(i * 0.021);
  } else {
    // corridor: forward along +x at 1.5 cm per frame
    pos = {1.6 + i * 0.015, -3.0 + 0.2 * std::sin(i * 0.004), 0.1 * std::sin(i * 0.007)};
    yaw = 8.0 * deg * std::sin(i * 0.006);
    pitch = -10.0 * deg + 3.0 * deg * std::sin(i * 0.011);
  }
  V3 f = {std::cos(yaw) * std::cos(pitch), std::sin(yaw) * std::cos(pitch), std::sin(pitch)};
  V3 right = unit(V3{f.y, -f.x, 0.0});
  V3 down = cross(f, right);
  double R[9] = {right.x, down.x, f.x, right.y, down.y, f.y, right.z, down.z, f.z};
  for (int a = 0; a < 3; ++a) {
    for (int b = 0; b < 3; ++b) T[a * 4 + b] = R[a * 3 + b];
  }
  T[3] = pos.x; T[7] = pos.y; T[11] = pos.z;
  T[12] = T[13] = T[14] = 0; T[15] = 1;
}

}  // namespace

extern "C" int sf_synth_create(const sf_synth_config *cfg, sf_synth **out) {
  if (!cfg || !out || cfg->cols <= 0 || cfg->rows <= 0) return 1;
  sf_synth *s = new sf_synth();
  s->cfg = *cfg;
  if (s->cfg.depth_scale <= 0) s->cfg.depth_scale = 1000.0f;
  build_scene(*s);
  *out = s;
  return 0;
}

extern "C" int sf_synth_destroy(sf_synth *s) { delete s; return 0; }

extern "C" int sf_synth_pose(const sf_synth *s, int i, double *pose) {
  if (!s || !pose) return 1;
  pose_at(*s, i, pose);
  return 0;
}

extern "C" int sf_synth_frame(const sf_synth *s, int i, uint16_t *depth, uint8_t *rgb,
                              uint8_t *mask, double *pose) {
  if (!s) return 1;
  const sf_synth_config &c = s->cfg;
  double T[16];
  pose_at(*s, i, T);
  if (pose) memcpy(pose, T, sizeof(T));
  V3 o = {T[3], T[7], T[11]};
  const uint64_t seed = c.seed;
  // rows are independent: render them on all host threads
  auto render_rows = [&](int v0, int v1) {
  for (int v = v0; v < v1; ++v)
    for (int u = 0; u < c.cols; ++u) {
      const size_t idx = (size_t)v * c.cols + u;
      V3 dc = {(u - c.cx) / c.fx, (v - c.cy) / c.fy, 1.0};
      V3 dw = {T[0] * dc.x + T[1] * dc.y + T[2] * dc.z, T[4] * dc.x + T[5] * dc.y + T[6] * dc.z,
               T[8] * dc.x + T[9] * dc.y + T[10] * dc.z};
      double t;
      int id;
      bool hit = intersect(*s, o, dw, t, id);
      uint64_t pk = (uint64_t)i * 0x9e3779b9ull + idx;
      double z = hit ? t : 0.0;
      if (depth) {
        uint16_t dmm = 0;
        if (hit && z > 0.05 && z < 10.0) {
          double sigma = 0.0012 + 0.0019 * (z - 0.4) * (z - 0.4);
          double zn = z + c.noise * sigma * gauss(key(seed, 1, pk, 0), key(seed, 2, pk, 0));
          double q = std::floor(zn * c.depth_scale + 0.5);
          if (q > 0 && q < 65535) dmm = (uint16_t)q;
          if (c.dropout > 0 && uni(key(seed, 3, pk, 0)) < c.dropout) dmm = 0;
        }
        depth[idx] = dmm;
      }
      V3 hp = add(o, scl(dw, t));
      if (rgb) {
        const double *base = (id < 0) ? s->room_rgb : s->prims[id].rgb;
        for (int q = 0; q < 3; ++q) {
          double n = grad_noise(seed + 101 * (q + 1), hp.x * 6.0, hp.y * 6.0, hp.z * 6.0) +
                     0.5 * grad_noise(seed + 313 * (q + 1), hp.x * 17.0, hp.y * 17.0, hp.z * 17.0);
          double val = base[q] * (0.75 + 0.5 * n);
          val = val < 0 ? 0 : (val > 255 ? 255 : val);
          rgb[3 * idx + q] = hit ? (uint8_t)val : 0;
        }
      }
      if (mask) {
        uint8_t cls = (hit && id >= 0) ? s->prims[id].cls : 0;
        if (c.label_flip > 0 && uni(key(seed, 4, pk, 0)) < c.label_flip)
          cls = (uint8_t)(key(seed, 5, pk, 0) % 81);
        mask[idx] = cls;
      }
    }
  };
  unsigned nt = std::thread::hardware_concurrency();
  nt = nt == 0 ? 1 : (nt > 64 ? 64 : nt);
  if ((int)nt > c.rows) nt = (unsigned)c.rows;
  std::vector<std::thread> pool;
  for (unsigned k = 1; k < nt; ++k)
    pool.emplace_back(render_rows, (int)((long)c.rows * k / nt), (int)((long)c.rows * (k + 1) / nt));
  render_rows(0, (int)((long)c.rows / nt));
  for (auto &th : pool) th.join();
  return 0;
}
