// Seeded synthetic RGB-D depth sequences (host C++).
//
// Stands in for the reference's capture layer (STAC/Util/z_yooji_frame_capture.cpp:
// uint16 millimetre depth maps, converted to metres with a 0.001 scale at :597)
// so that benchmarks and tests have repeatable input.  A scene is 3-6 spheres
// and yawed boxes (radius / half-size 5-15 cm) resting on a ground plane; the
// camera orbits the scene centre on a horizontal circle of radius 0.9 m at a
// height that puts it 1 m from the centre, 0.5 deg per frame, with Gaussian
// jitter.  Depth is the analytic ray hit, plus Kinect-style axial noise
// sigma(z) = 0.0012 + 0.0019 (z - 0.4)^2 m, dropout (i.i.d. pixels or 8x8
// blobs), an optional far cut-off, and uint16 millimetre quantisation.
//
// Determinism: every random draw is a counter-based hash of (seed, frame,
// pixel, stream), so the output does not depend on threading.  Normal deviates
// are Irwin-Hall sums of 12 uniforms (mean 0, variance 1).  Fixtures that are
// checked on another host store their input frames, so no test relies on
// libm's sin/cos rounding identically across hosts.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "vs_synth.h"

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
inline uint64_t key(uint64_t seed, uint64_t a, uint64_t b, uint64_t c) {
  return mix64(seed ^ mix64(a ^ mix64(b ^ mix64(c))));
}
inline double uniform(uint64_t k) { return (double)(mix64(k) >> 11) * (1.0 / 9007199254740992.0); }
inline double normal(uint64_t k) {
  double s = 0;
  for (int i = 0; i < 12; i++) s += uniform(k + 0x1000003ull * (uint64_t)(i + 1));
  return s - 6.0;
}

struct Prim {
  int type;  // 0 sphere, 1 box
  double c[3];
  double r;        // sphere radius
  double h[3];     // box half extents
  double yaw;      // box yaw about the vertical axis
};

struct Scene {
  std::vector<Prim> prims;
  double centre[3];
};

Scene make_scene(uint64_t seed) {
  Scene s;
  int n = 3 + (int)(mix64(key(seed, 1, 0, 0)) % 4);
  s.centre[0] = 0;
  s.centre[1] = 0.10;
  s.centre[2] = 0;
  for (int i = 0; i < n; i++) {
    Prim p;
    std::memset(&p, 0, sizeof(p));
    p.type = (int)(mix64(key(seed, 2, i, 0)) & 1);
    double ang = 2.0 * M_PI * uniform(key(seed, 3, i, 0));
    double rad = 0.28 * std::sqrt(uniform(key(seed, 4, i, 0)));
    double size = 0.05 + 0.10 * uniform(key(seed, 5, i, 0));
    p.c[0] = rad * std::cos(ang);
    p.c[2] = rad * std::sin(ang);
    if (p.type == 0) {
      p.r = size;
      p.c[1] = size;
    } else {
      p.h[0] = size;
      p.h[1] = 0.05 + 0.10 * uniform(key(seed, 6, i, 0));
      p.h[2] = 0.05 + 0.10 * uniform(key(seed, 7, i, 0));
      p.c[1] = p.h[1];
      p.yaw = M_PI * uniform(key(seed, 8, i, 0));
    }
    s.prims.push_back(p);
  }
  return s;
}

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
inline void norm3(double* a) {
  double l = std::sqrt(dot3(a, a));
  a[0] /= l;
  a[1] /= l;
  a[2] /= l;
}

// nearest positive hit along o + t d (t measured in units of d)
double hit(const Scene& s, const double* o, const double* d) {
  double best = 1e30;
  if (d[1] < 0) {
    double t = -o[1] / d[1];
    if (t > 0 && t < best) best = t;
  }
  for (const Prim& p : s.prims) {
    if (p.type == 0) {
      double oc[3] = {o[0] - p.c[0], o[1] - p.c[1], o[2] - p.c[2]};
      double a = dot3(d, d), b = 2 * dot3(d, oc), c = dot3(oc, oc) - p.r * p.r;
      double disc = b * b - 4 * a * c;
      if (disc < 0) continue;
      double sq = std::sqrt(disc);
      double t = (-b - sq) / (2 * a);
      if (t <= 0) t = (-b + sq) / (2 * a);
      if (t > 0 && t < best) best = t;
    } else {
      double cy = std::cos(p.yaw), sy = std::sin(p.yaw);
      double ol[3], dl[3];
      double oc[3] = {o[0] - p.c[0], o[1] - p.c[1], o[2] - p.c[2]};
      // rotate into the box frame (inverse yaw about y)
      ol[0] = cy * oc[0] - sy * oc[2];
      ol[1] = oc[1];
      ol[2] = sy * oc[0] + cy * oc[2];
      dl[0] = cy * d[0] - sy * d[2];
      dl[1] = d[1];
      dl[2] = sy * d[0] + cy * d[2];
      double t0 = -1e30, t1 = 1e30;
      bool miss = false;
      for (int k = 0; k < 3; k++) {
        if (std::fabs(dl[k]) < 1e-15) {
          if (std::fabs(ol[k]) > p.h[k]) miss = true;
          continue;
        }
        double a = (-p.h[k] - ol[k]) / dl[k], b = (p.h[k] - ol[k]) / dl[k];
        if (a > b) std::swap(a, b);
        t0 = std::max(t0, a);
        t1 = std::min(t1, b);
      }
      if (miss || t0 > t1) continue;
      double t = t0 > 0 ? t0 : t1;
      if (t > 0 && t < best) best = t;
    }
  }
  return best;
}

// camera k pose: rotation camera->scene (columns x, y, z) and position
void camera_pose(const vs_synth_config* c, const Scene& s, int k, double R[9], double pos[3]) {
  uint64_t sd = c->seed;
  double phi = (c->orbit_start_deg + c->orbit_step_deg * k) * M_PI / 180.0;
  phi += c->jitter_deg * M_PI / 180.0 * normal(key(sd, 100, k, 0));
  double rad = c->orbit_radius;
  double h = std::sqrt(std::max(0.0, c->view_distance * c->view_distance - rad * rad));
  pos[0] = s.centre[0] + rad * std::sin(phi) + c->jitter_m * normal(key(sd, 101, k, 0));
  pos[1] = s.centre[1] + h + c->jitter_m * normal(key(sd, 102, k, 0));
  pos[2] = s.centre[2] + rad * std::cos(phi) + c->jitter_m * normal(key(sd, 103, k, 0));
  double tgt[3];
  for (int i = 0; i < 3; i++) tgt[i] = s.centre[i] + c->jitter_m * normal(key(sd, 104 + i, k, 0));
  double z[3] = {tgt[0] - pos[0], tgt[1] - pos[1], tgt[2] - pos[2]};
  norm3(z);
  double down[3] = {0, -1, 0};
  double x[3], y[3];
  cross3(down, z, x);
  norm3(x);
  cross3(z, x, y);
  // small roll jitter about the optical axis
  double roll = c->jitter_deg * M_PI / 180.0 * normal(key(sd, 110, k, 0));
  double cr = std::cos(roll), sr = std::sin(roll);
  double xr[3], yr[3];
  for (int i = 0; i < 3; i++) {
    xr[i] = cr * x[i] + sr * y[i];
    yr[i] = -sr * x[i] + cr * y[i];
  }
  for (int i = 0; i < 3; i++) {
    R[i * 3 + 0] = xr[i];
    R[i * 3 + 1] = yr[i];
    R[i * 3 + 2] = z[i];
  }
}

}  // namespace

extern "C" {

void vs_synth_default(vs_synth_config* c, int width, int height) {
  std::memset(c, 0, sizeof(*c));
  c->width = width;
  c->height = height;
  c->fx = c->fy = 525.0f;
  c->cx = 0.5f * width - 0.5f;
  c->cy = 0.5f * height - 0.5f;
  c->n_frames = 30;
  c->seed = 1;
  c->orbit_radius = 0.9;
  c->view_distance = 1.0;
  c->orbit_start_deg = 0;
  c->orbit_step_deg = 0.5;
  c->jitter_deg = 0.05;
  c->jitter_m = 0.001;
  c->noise = 1;
  c->dropout_iid = 0.0;
  c->dropout_blob = 0.0;
  c->max_depth = 0.0;
  c->threads = 0;
}

static int generate(const vs_synth_config* c, uint16_t* depth, uint8_t* rgb, double* T_gc, double* centre_cam0);

int vs_synth_generate(const vs_synth_config* c, uint16_t* depth, double* T_gc, double* centre_cam0) {
  return generate(c, depth, nullptr, T_gc, centre_cam0);
}

int vs_synth_generate_rgb(const vs_synth_config* c, uint16_t* depth, uint8_t* rgb, double* T_gc,
                          double* centre_cam0) {
  if (!rgb) return -1;
  return generate(c, depth, rgb, T_gc, centre_cam0);
}

// colour of a surface point (scene frame): a smooth procedural texture, every
// channel in 30..230 so a hit never reads as "no colour"
static void surface_rgb(const double* P, uint8_t out[3]) {
  const double f[3] = {9.0 * P[0], 7.0 * P[2] + 1.0, 11.0 * P[1] + 2.0};
  for (int k = 0; k < 3; k++) out[k] = (uint8_t)(30.0 + 200.0 * (0.5 + 0.5 * std::sin(f[k])) + 0.5);
}

static int generate(const vs_synth_config* c, uint16_t* depth, uint8_t* rgb, double* T_gc, double* centre_cam0) {
  if (!c || c->width <= 0 || c->height <= 0 || c->n_frames <= 0) return -1;
  Scene s = make_scene(c->seed);
  const int W = c->width, H = c->height, N = c->n_frames;
  // global frame = camera 0 (the reference starts tracking from the identity)
  double R0[9], p0[3];
  camera_pose(c, s, 0, R0, p0);
  if (centre_cam0) {
    double d[3] = {s.centre[0] - p0[0], s.centre[1] - p0[1], s.centre[2] - p0[2]};
    for (int i = 0; i < 3; i++) centre_cam0[i] = R0[0 * 3 + i] * d[0] + R0[1 * 3 + i] * d[1] + R0[2 * 3 + i] * d[2];
  }
  unsigned nt = c->threads > 0 ? (unsigned)c->threads : std::max(1u, std::thread::hardware_concurrency());
  for (int k = 0; k < N; k++) {
    double R[9], pos[3];
    camera_pose(c, s, k, R, pos);
    if (T_gc) {
      // T_gc = inv(T_s<-ck) * T_s<-c0 ; rows of R^T
      double A[16] = {0}, B[16] = {0}, O[16];
      for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) A[i * 4 + j] = R[j * 3 + i];
        A[i * 4 + 3] = -(R[0 * 3 + i] * pos[0] + R[1 * 3 + i] * pos[1] + R[2 * 3 + i] * pos[2]);
        for (int j = 0; j < 3; j++) B[i * 4 + j] = R0[i * 3 + j];
        B[i * 4 + 3] = p0[i];
      }
      A[15] = B[15] = 1;
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
          double acc = 0;
          for (int q = 0; q < 4; q++) acc += A[i * 4 + q] * B[q * 4 + j];
          O[i * 4 + j] = acc;
        }
      std::memcpy(T_gc + 16 * (size_t)k, O, sizeof(O));
    }
    uint16_t* out = depth + (size_t)k * W * H;
    uint8_t* col = rgb ? rgb + (size_t)k * 3 * W * H : nullptr;
    auto rows = [&](int r0, int r1) {
      for (int v = r0; v < r1; v++)
        for (int u = 0; u < W; u++) {
          double dc[3] = {(u - c->cx) / c->fx, (v - c->cy) / c->fy, 1.0};
          double d[3] = {R[0] * dc[0] + R[1] * dc[1] + R[2] * dc[2], R[3] * dc[0] + R[4] * dc[1] + R[5] * dc[2],
                         R[6] * dc[0] + R[7] * dc[1] + R[8] * dc[2]};
          double t = hit(s, pos, d);
          double z = (t < 1e29) ? t : 0.0;
          uint64_t pk = (uint64_t)v * W + u;
          if (col) {
            uint8_t cc[3] = {0, 0, 0};
            if (t < 1e29) {
              const double P[3] = {pos[0] + t * d[0], pos[1] + t * d[1], pos[2] + t * d[2]};
              surface_rgb(P, cc);
            }
            for (int ch = 0; ch < 3; ch++) col[(size_t)ch * W * H + pk] = cc[ch];
          }
          if (z > 0 && c->noise) {
            double sig = 0.0012 + 0.0019 * (z - 0.4) * (z - 0.4);
            z += sig * normal(key(c->seed, 200, k, pk));
          }
          if (c->max_depth > 0 && z > c->max_depth) z = 0;
          if (c->dropout_iid > 0 && uniform(key(c->seed, 300, k, pk)) < c->dropout_iid) z = 0;
          double mm = std::floor(z * 1000.0 + 0.5);
          if (!(mm > 0)) mm = 0;
          if (mm > 65535) mm = 0;
          out[pk] = (uint16_t)mm;
        }
    };
    std::vector<std::thread> th;
    int chunk = (H + (int)nt - 1) / (int)nt;
    for (unsigned i = 0; i < nt; i++) {
      int r0 = (int)i * chunk, r1 = std::min(H, r0 + chunk);
      if (r0 < r1) th.emplace_back(rows, r0, r1);
    }
    for (auto& t : th) t.join();
    if (c->dropout_blob > 0) {
      int nb = (int)std::floor(c->dropout_blob * W * H / 64.0 + 0.5);
      for (int b = 0; b < nb; b++) {
        int x0 = (int)(uniform(key(c->seed, 400, k, 2 * b)) * (W - 7));
        int y0 = (int)(uniform(key(c->seed, 400, k, 2 * b + 1)) * (H - 7));
        for (int y = y0; y < y0 + 8 && y < H; y++)
          for (int x = x0; x < x0 + 8 && x < W; x++) out[(size_t)y * W + x] = 0;
      }
    }
  }
  return 0;
}

}  // extern "C"
