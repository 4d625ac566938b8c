// Golden-vector harness around the reference's own sequential 7-point
// diffusion (examples/diffusion-benchmark/baseline.cc:22-49, coefficients
// diffusion3d.h:45-57, initial field diffusion3d.cc:14-40).  Test
// infrastructure only: it is compiled against the reference sources where
// they lie and writes, for an n^3 grid and `count` steps,
//   <out>.init.f32   the initial field (raw little-endian float32)
//   <out>.final.f32  the field after `count` steps (raw float32)
//   <out>.coef.txt   ce cw cn cs ct cb cc as C99 hex floats
// Usage: ref_diffusion_harness <n> <count> <out-prefix>
#include <cstdio>
#include <cstdlib>
#include <string>
#include "baseline.h"

namespace {
class Harness : public diffusion3d::Baseline {
 public:
  Harness(int n) : Baseline(n, n, n) {}
  void Go(int count, const std::string &out) {
    InitializeBenchmark();
    Write(out + ".init.f32");
    RunKernel(count);
    Write(out + ".final.f32");
    FILE *f = fopen((out + ".coef.txt").c_str(), "w");
    fprintf(f, "%a %a %a %a %a %a %a\n", ce_, cw_, cn_, cs_, ct_, cb_, cc_);
    fclose(f);
    FinalizeBenchmark();
  }
  void Write(const std::string &path) {
    FILE *f = fopen(path.c_str(), "wb");
    fwrite(f1_, sizeof(REAL), (size_t)nx_ * ny_ * nz_, f);
    fclose(f);
  }
};
}  // namespace

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s n count out-prefix\n", argv[0]);
    return 2;
  }
  Harness h(atoi(argv[1]));
  h.Go(atoi(argv[2]), argv[3]);
  return 0;
}
