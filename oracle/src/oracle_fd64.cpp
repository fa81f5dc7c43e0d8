// oracle_fd64.cpp -- TEST INFRASTRUCTURE.  A float64 restatement of the
// single-layer sphere frame (the path the adjoint differentiates) for finite
// differences: primary rays (embree_renderer.cpp:375-386, 1399-1414), sphere
// hits, shadeHit's sphere branch (hit_shader.hpp:311-345), shadeLocal's POV
// branch (shading.hpp:76-192), hard shadows (secondary_rays.hpp:118-134),
// legacy and enhanced AO (ambient_occlusion.hpp:33-57, 171-267),
// aoApplyFactors without bent normal / multibounce (ao_shade.hpp:80-117), fog
// (fog.cpp:17-36), box downsample (image_ops.cpp:9-35) and assumed gamma
// (image_ops.cpp:37-46), every quantity in double.
//
// Visibility record: a call with record = 1 traces every ray by brute force
// over the spheres and writes, per hi-res sample, the primary sphere and root,
// the frame-from-normal branch, each light's lit / shadowed state and each AO
// sample's grazing test and occluder (sphere and root).  A call with
// record = 0 evaluates the image with that visibility held fixed, so central
// differences of it are smooth in every parameter -- the derivative the
// adjoint computes.  AO sample coordinates come from the same float tea2 /
// low-discrepancy streams as the renderer.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

struct D3 {
  double x, y, z;
};
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline D3 normalize(D3 a) {
  const double l = std::sqrt(dot(a, a));
  return l > 0.0 ? a * (1.0 / l) : a;
}
inline D3 safeNormalize(D3 a, D3 fb) {
  const double d = dot(a, a);
  if (d < 1.0e-18) return fb;
  return a * (1.0 / std::sqrt(d));
}

// secondary_rays.hpp:51-61 (the sample streams stay in float / u32)
inline void tea2(uint32_t& v0, uint32_t& v1) {
  uint32_t sum = 0;
  for (int i = 0; i < 8; ++i) {
    sum += 0x9E3779B9u;
    v0 += ((v1 << 4) + 0xA341316Cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xC8013EA4u);
    v1 += ((v0 << 4) + 0xAD90777Du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7E95761Eu);
  }
}
inline float u32ToUnorm(uint32_t u) { return (u >> 8) * 0x1.0p-24f; }
inline float radicalInverse2(uint32_t bits) {
  bits = (bits << 16) | (bits >> 16);
  bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
  bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
  bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
  bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
  return static_cast<float>(bits) * 0x1.0p-32f;
}

}  // namespace

extern "C" {

// Parameters of the float64 frame (every real in double).
struct fd64_desc {
  int32_t width, height, ss, ortho;
  double cam_pos[3], cam_dir[3], cam_up[3];
  double cam_height, cam_fovy;
  double clip_near, clip_far;
  double ambient_color[3], background[3];
  int32_t n_lights, shadows, ao_samples, ao_multiscale;
  double light_dir[4][3], light_color[4][3], light_intensity[4];
  int32_t light_highlight[4];
  double ao_distance, ao_intensity, ao_falloff_power, ao_diffuse_factor;
  int32_t ao_low_discrepancy, ao_enhanced, fog_on, transparent_bg;
  double fog_start, fog_end, fog_color[3];
  double gamma, specular_scale;
  double mat[9];  // ambient diffuse specular roughness brilliance phong phong_size reflection emission
  int32_t metallic, pad;
  // the frame is a window of a larger frame: the per-pixel sample streams are
  // seeded with the window's pixels' coordinates in that frame (seed_w wide;
  // 0 = this frame is the whole frame)
  int32_t seed_x0, seed_y0, seed_w, pad2;
};

// Visibility record entries per hi-res sample.
int32_t oracle_fd64_vis_stride(int32_t ao_samples) { return 2 + 4 + ao_samples; }

}  // extern "C"

namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();

struct Roots {
  bool hit;
  double tf, tb;
};
// isectSphere in double: roots of |o + t d - c| = r (perpendicular form)
inline Roots sphereRoots(D3 o, D3 d, const double* s) {
  const D3 c0{s[0] - o.x, s[1] - o.y, s[2] - o.z};
  const double rd2 = 1.0 / dot(d, d);
  const double proj = dot(c0, d) * rd2;
  const D3 perp = c0 - d * proj;
  const double l2 = dot(perp, perp), r2 = s[3] * s[3];
  Roots r{l2 <= r2, 0.0, 0.0};
  const double td = std::sqrt(std::fmax(r2 - l2, 0.0) * rd2);
  r.tf = proj - td;
  r.tb = proj + td;
  return r;
}

// closest sphere hit in [tn, tf]; returns code prim*2 + root or -1
inline int64_t closest(const double* sph, uint64_t n, D3 o, D3 d, double tn, double tfar, double& tOut) {
  int64_t best = -1;
  double bt = tfar;
  for (uint64_t i = 0; i < n; ++i) {
    const Roots r = sphereRoots(o, d, sph + 4 * i);
    if (!r.hit) continue;
    double t;
    int root;
    if (r.tf >= tn && r.tf <= bt) { t = r.tf; root = 0; }
    else if (r.tb >= tn && r.tb <= bt) { t = r.tb; root = 1; }
    else continue;
    if (best < 0 || t < bt) {
      bt = t;
      best = int64_t(i) * 2 + root;
    }
  }
  tOut = bt;
  return best;
}

inline bool anyHit(const double* sph, uint64_t n, D3 o, D3 d, double tn, double tfar) {
  for (uint64_t i = 0; i < n; ++i) {
    const Roots r = sphereRoots(o, d, sph + 4 * i);
    if (!r.hit) continue;
    if ((r.tf >= tn && r.tf <= tfar) || (r.tb >= tn && r.tb <= tfar)) return true;
  }
  return false;
}

inline double rootOf(const double* sph, int64_t code, D3 o, D3 d) {
  const Roots r = sphereRoots(o, d, sph + 4 * (code >> 1));
  return (code & 1) ? r.tb : r.tf;
}

struct Cam {
  D3 pos, dir, right, up;
  double halfW, halfH, pHalfW, pHalfH;
};

void renderRows(const fd64_desc& d, const double* sph, const double* col, uint64_t n, int32_t* vis, int record,
                double* hi, const Cam& cam, int row0, int row1) {
  const int W = d.width * d.ss, H = d.height * d.ss;
  const int stride = oracle_fd64_vis_stride(d.ao_samples);
  const double K = 0x1.0fp-21;
  D3 Ls[4], Lc[4];
  for (int l = 0; l < d.n_lights; ++l) {
    Ls[l] = normalize(D3{-d.light_dir[l][0], -d.light_dir[l][1], -d.light_dir[l][2]});
    Lc[l] = D3{d.light_color[l][0] * d.light_intensity[l], d.light_color[l][1] * d.light_intensity[l],
               d.light_color[l][2] * d.light_intensity[l]};
  }
  const double* m = d.mat;
  for (int py = row0; py < row1; ++py)
    for (int px = 0; px < W; ++px) {
      int32_t* v = vis + (size_t(py) * W + px) * stride;
      double* outp = hi + (size_t(py) * W + px) * 4;
      const double vv = 1.0 - 2.0 * (py + 0.5) / H;
      const double uu = 2.0 * (px + 0.5) / W - 1.0;
      D3 org, rd;
      if (d.ortho) {
        org = cam.pos + cam.right * (uu * cam.halfW) + cam.up * (vv * cam.halfH);
        rd = cam.dir;
      } else {
        org = cam.pos;
        rd = normalize(cam.dir + cam.right * (uu * cam.pHalfW) + cam.up * (vv * cam.pHalfH));
      }
      double tn = 0.0, tfar = kInf;
      if (!(d.clip_near <= -kInf && d.clip_far >= kInf)) {
        const double cosr = dot(rd, cam.dir);
        if (!(cosr <= 1.0e-6)) {
          if (d.clip_near > 0.0) tn = d.clip_near / cosr;
          if (d.clip_far < kInf) tfar = d.clip_far / cosr;
        }
      }
      int64_t code;
      double t = 0.0;
      if (record) {
        code = closest(sph, n, org, rd, tn, tfar, t);
        v[0] = int32_t(code);
      } else {
        code = v[0];
        if (code >= 0) t = rootOf(sph, code, org, rd);
      }
      const double cov = d.transparent_bg ? 0.0 : 1.0;
      if (code < 0) {
        outp[0] = d.background[0] * cov;
        outp[1] = d.background[1] * cov;
        outp[2] = d.background[2] * cov;
        outp[3] = cov;
        continue;
      }
      const uint64_t k = uint64_t(code >> 1);
      const double* s = sph + 4 * k;
      const D3 P = org + rd * t;
      const D3 Ng = P - D3{s[0], s[1], s[2]};
      D3 N = normalize(Ng);
      if (dot(N, rd) > 0.0) N = N * -1.0;
      const D3 V = normalize(rd * -1.0);
      const double dirMax = std::fmax(std::fabs(rd.x), std::fmax(std::fabs(rd.y), std::fabs(rd.z)));
      const double eps =
          std::fmax(std::fmax(std::fabs(P.x), std::fabs(P.y)), std::fmax(std::fabs(P.z), dirMax * t)) * K;
      D3 ng = dot(Ng, N) < 0.0 ? Ng * -1.0 : Ng;
      ng = safeNormalize(ng, N);
      const D3 O = P + ng * eps;
      const D3 C{col[3 * k], col[3 * k + 1], col[3 * k + 2]};
      // AO
      double openness = 1.0;
      if (d.ao_samples > 0) {
        bool seed0;
        if (record) {
          seed0 = std::fabs(N.x) < std::fabs(N.y);
          v[1] = seed0 ? 1 : 0;
        } else {
          seed0 = v[1] != 0;
        }
        const D3 sd = seed0 ? D3{0.0, N.z, -N.y} : D3{-N.z, 0.0, N.x};
        const D3 ft = safeNormalize(sd, D3{1.0, 0.0, 0.0});
        const D3 fb = cross(N, ft);
        const double R = d.ao_distance;
        double radius[3], weight[3];
        int KS;
        if (d.ao_enhanced && d.ao_multiscale) {
          KS = 3;
          radius[0] = 0.08 * R; radius[1] = 0.30 * R; radius[2] = R;
          weight[0] = 0.55; weight[1] = 0.35; weight[2] = 0.10;
        } else {
          KS = 1;
          radius[0] = R;
          weight[0] = 1.0;
        }
        const uint32_t sx = uint32_t(px + d.seed_x0), sy = uint32_t(py + d.seed_y0);
        const uint32_t base = sx + sy * uint32_t(d.seed_w > 0 ? d.seed_w : W);
        float cpx = 0.0f, cpy = 0.0f;
        if (d.ao_enhanced && d.ao_low_discrepancy) {
          uint32_t c0 = sx + 1u, c1 = sy + 1u;
          tea2(c0, c1);
          cpx = u32ToUnorm(c0);
          cpy = u32ToUnorm(c1);
        }
        double obs = 0.0;
        for (int i = 0; i < d.ao_samples; ++i) {
          float u1, u2;
          if (d.ao_enhanced && d.ao_low_discrepancy) {
            u1 = float(i) / float(d.ao_samples) + cpx;
            u2 = radicalInverse2(uint32_t(i)) + cpy;
            if (u1 >= 1.0f) u1 -= 1.0f;
            if (u2 >= 1.0f) u2 -= 1.0f;
          } else {
            uint32_t s0 = base, s1 = uint32_t(i);
            tea2(s0, s1);
            u1 = u32ToUnorm(s0);
            u2 = u32ToUnorm(s1);
          }
          const double phi = 6.2831853072 * double(u1);
          const double rr = std::sqrt(double(u2));
          const double cz = std::sqrt(std::fmax(0.0, 1.0 - double(u2)));
          const D3 dir = ft * (std::cos(phi) * rr) + fb * (std::sin(phi) * rr) + N * cz;
          int32_t& a = v[6 + i];
          if (record) {
            if (dot(dir, N) < 0.01) {
              a = -2;
            } else {
              double th;
              a = int32_t(closest(sph, n, O, dir, eps, R, th));
            }
          }
          if (a == -2) {
            obs += 1.0;
            continue;
          }
          if (a < 0) continue;
          if (!d.ao_enhanced) {
            obs += 1.0;
            continue;
          }
          const double th = rootOf(sph, a, O, dir);
          for (int q = 0; q < KS; ++q)
            if (th < radius[q]) {
              double fk = 1.0;
              if (d.ao_falloff_power > 0.0) fk = std::pow(std::fmax(1.0 - th / radius[q], 0.0), d.ao_falloff_power);
              obs += weight[q] * fk;
            }
        }
        openness = 1.0 - obs / d.ao_samples;
      }
      const double aoF = d.ao_samples > 0 ? 1.0 - d.ao_intensity * (1.0 - openness) : 1.0;
      const double diffuseAo =
          (d.ao_samples > 0 && d.ao_diffuse_factor > 0.0) ? 1.0 - d.ao_diffuse_factor * (1.0 - openness) : 1.0;
      D3 out{m[8] * C.x + aoF * m[0] * C.x * d.ambient_color[0], m[8] * C.y + aoF * m[0] * C.y * d.ambient_color[1],
             m[8] * C.z + aoF * m[0] * C.z * d.ambient_color[2]};
      double ex = 1.0 / std::fmax(m[3], 1e-6);
      ex = std::fmin(std::fmax(ex, 1.0), 1.0e6);
      for (int l = 0; l < d.n_lights; ++l) {
        const D3 L = Ls[l];
        const double ndl = dot(N, L);
        int32_t& lc = v[2 + l];
        if (record) {
          if (!(ndl > 0.0)) lc = 0;
          else lc = (d.shadows && anyHit(sph, n, O, L, eps, kInf)) ? 2 : 1;
        }
        if (lc == 0) continue;
        const double sf = lc == 2 ? 0.0 : 1.0;
        const D3 lcol = Lc[l] * sf;
        double dd;
        if (m[4] == 1.0) dd = ndl;
        else if (m[4] == 0.0) dd = 1.0;
        else dd = std::pow(ndl, m[4]);
        const double dk = m[1] * dd * diffuseAo;
        out.x += dk * C.x * lcol.x;
        out.y += dk * C.y * lcol.y;
        out.z += dk * C.z * lcol.z;
        if (!d.light_highlight[l]) continue;
        D3 hl;
        if (d.metallic) {
          const double c = std::fmin(ndl, 1.0);
          const double x = std::acos(c) * 0.63661977;
          double f = 0.014567225 / ((x - 1.12) * (x - 1.12)) - 0.011612903;
          f = std::fmin(std::fmax(f, 0.0), 1.0);
          hl = D3{lcol.x * (f + (1.0 - f) * C.x), lcol.y * (f + (1.0 - f) * C.y), lcol.z * (f + (1.0 - f) * C.z)};
        } else {
          hl = lcol;
        }
        double specW = 0.0;
        if (m[2] > 0.0) {
          const D3 Hh = normalize(L + V);
          const double nh = dot(N, Hh);
          if (nh > 0.0) specW += m[2] * std::pow(nh, ex);
        }
        if (m[5] > 0.0) {
          const D3 Rr = N * (2.0 * ndl) - L;
          const double rv = dot(Rr, V);
          if (rv > 0.0 && (m[6] < 60.0 || rv > 0.0008)) specW += m[5] * std::pow(rv, m[6]);
        }
        if (specW > 0.0) {
          const double sc = specW * d.specular_scale;
          out = out + hl * sc;
        }
      }
      if (m[7] > 0.0) out = out + D3{d.background[0], d.background[1], d.background[2]} * m[7];
      double a4 = 1.0;
      if (d.fog_on) {
        const double z = t * dot(rd, cam.dir);
        if (z > 0.0) {
          double f;
          const double den = d.fog_end - d.fog_start;
          if (den <= 0.0) f = z < d.fog_end ? 1.0 : 0.0;
          else f = std::fmin(std::fmax((d.fog_end - z) / den, 0.0), 1.0);
          if (d.transparent_bg) {
            a4 *= f;
          } else {
            out.x = d.fog_color[0] * (1.0 - f) + out.x * f;
            out.y = d.fog_color[1] * (1.0 - f) + out.y * f;
            out.z = d.fog_color[2] * (1.0 - f) + out.z * f;
          }
        }
      }
      outp[0] = out.x;
      outp[1] = out.y;
      outp[2] = out.z;
      outp[3] = a4;
    }
}

}  // namespace

extern "C" int oracle_fd64_render(const fd64_desc* dp, const double* sph, const double* col, uint64_t n,
                                  int32_t* vis, int record, double* out, int threads) {
  const fd64_desc& d = *dp;
  if (d.width <= 0 || d.height <= 0 || d.ss < 1 || d.n_lights > 4 || d.ao_samples < 0) return 1;
  const int W = d.width * d.ss, H = d.height * d.ss;
  Cam cam;
  // computeCameraBasis (embree_renderer.cpp:375-386)
  cam.pos = D3{d.cam_pos[0], d.cam_pos[1], d.cam_pos[2]};
  cam.dir = normalize(D3{d.cam_dir[0], d.cam_dir[1], d.cam_dir[2]});
  cam.right = normalize(cross(cam.dir, D3{d.cam_up[0], d.cam_up[1], d.cam_up[2]}));
  cam.up = normalize(cross(cam.right, cam.dir));
  const double aspect = double(W) / double(H);
  cam.halfH = d.cam_height * 0.5;
  cam.halfW = cam.halfH * aspect;
  cam.pHalfH = std::tan(d.cam_fovy * 0.017453292519943295 * 0.5);
  cam.pHalfW = cam.pHalfH * aspect;
  std::vector<double> hi(size_t(W) * H * 4);
  if (threads < 1) threads = 1;
  std::vector<std::thread> pool;
  for (int k = 0; k < threads; ++k) {
    const int r0 = H * k / threads, r1 = H * (k + 1) / threads;
    pool.emplace_back(renderRows, std::cref(d), sph, col, n, vis, record, hi.data(), std::cref(cam), r0, r1);
  }
  for (auto& th : pool) th.join();
  // box downsample + assumed gamma
  const int ss = d.ss;
  for (int oy = 0; oy < d.height; ++oy)
    for (int ox = 0; ox < d.width; ++ox) {
      double a[4] = {0.0, 0.0, 0.0, 0.0};
      for (int dy = 0; dy < ss; ++dy)
        for (int dx = 0; dx < ss; ++dx) {
          const double* c = &hi[(size_t(oy * ss + dy) * W + size_t(ox * ss + dx)) * 4];
          for (int q = 0; q < 4; ++q) a[q] += c[q];
        }
      double* o = out + (size_t(oy) * d.width + ox) * 4;
      for (int q = 0; q < 4; ++q) o[q] = a[q] / double(ss * ss);
      if (!(std::fabs(d.gamma - 1.0) <= 1.0e-4))
        for (int q = 0; q < 3; ++q) o[q] = o[q] > 0.0 ? std::pow(o[q], d.gamma) : 0.0;
    }
  return 0;
}
