// Host check of the MIP condition's shortcut (shocovox_gb300/csrc/svo_lod.h): lod_reads_mip must
// equal the reference's f32 evaluation (lod_reads_mip_exact) on random and near-boundary cases.
// Usage: lod_condition_check <cases>; prints "OK <cases> <decided by the shortcut>" or the first
// mismatch.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../shocovox_gb300/csrc/svo_lod.h"

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  const float sizes[] = {16.0f, 64.0f, 512.0f, 4096.0f, 65536.0f};
  long shortcut = 0;
  for (long i = 0; i < n; ++i) {
    const float S = sizes[rng() % 5];
    float o[3], p[3];
    for (int k = 0; k < 3; ++k) {
      o[k] = (float)((u01(rng) * 5.0 - 2.0) * S);
      p[k] = (float)(u01(rng) * S);
    }
    if (rng() % 64 == 0) o[rng() % 3] = p[rng() % 3];  // shared coordinates
    float level = (float)((int)(rng() % 15) - 2);        // drifted levels below 1 included
    if (rng() % 16 == 0) level = (float)(u01(rng) * 20.0 - 4.0);
    const double dx = (double)o[0] - p[0], dy = (double)o[1] - p[1], dz = (double)o[2] - p[2];
    const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
    float vd;
    switch (rng() % 8) {
      case 0: vd = (float)std::exp(u01(rng) * 30.0 - 10.0); break;  // log-uniform 4.5e-5 .. 5e8
      case 1: vd = FLT_MAX; break;
      case 2: vd = (float)(rng() % 4 == 0 ? 0.0 : (rng() % 2 ? 1e-40 : -3.0)); break;
      case 3: vd = level != 0.0f ? (float)((d + 1.7320508 * level * (u01(rng) * 2.0 - 1.0)) / level) : 1.0f;
        break;  // inside the ambiguous band
      default: {  // within a few parts in 2^16 of the boundary |o - p| / level
        const double t = (u01(rng) * 2.0 - 1.0) * std::ldexp(1.0, -(int)(rng() % 24));
        vd = level != 0.0f ? (float)(d / level * (1.0 + t)) : 1.0f;
      }
    }
    if (rng() % 512 == 0) o[rng() % 3] = (rng() % 2) ? NAN : INFINITY;
    const bool a = svo::lod_reads_mip(o[0], o[1], o[2], p[0], p[1], p[2], level, vd);
    const bool b = svo::lod_reads_mip_exact(o[0], o[1], o[2], p[0], p[1], p[2], level, vd);
    if (a != b) {
      printf("MISMATCH o=(%a, %a, %a) p=(%a, %a, %a) level=%a vd=%a: shortcut %d exact %d\n", o[0], o[1], o[2], p[0],
             p[1], p[2], level, vd, a, b);
      return 1;
    }
    // how often the shortcut decided (the same tests as in the header)
    if (level > 0.0f && vd > 0.0f) {
      const float ex = o[0] - p[0], ey = o[1] - p[1], ez = o[2] - p[2];
      const float r2 = (ex * ex + ey * ey) + ez * ez;
      const float k = 1.7321f * (level + 0x1p-20f * (((fabsf(p[0]) + fabsf(p[1])) + fabsf(p[2])) + level));
      const float lv = level * vd;
      const float lo = lv * (1.0f - 0x1p-16f) - k, hi = lv * (1.0f + 0x1p-16f) + k;
      if ((lo > 0.0f && r2 < (lo * lo) * (1.0f - 0x1p-16f)) || r2 > (hi * hi) * (1.0f + 0x1p-16f)) ++shortcut;
    }
  }
  printf("OK %ld %ld\n", n, shortcut);
  return 0;
}
