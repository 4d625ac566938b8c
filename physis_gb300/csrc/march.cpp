// Work decomposition shared by the z-marching kernels (stencil7.cu,
// himeno19.cu): the choice of z-chunk length for the chunk-major schedule.
#include "ps_internal.h"

namespace psg {

int choose_zchunk(int tiles, int nz, int resident) {
  return choose_zchunk_overhead(tiles, nz, resident, 1);
}

int choose_zchunk_overhead(int tiles, int nz, int resident, int overhead) {
  if (nz <= 1 || tiles <= 0 || resident <= 0) return nz > 0 ? nz : 1;
  int best_len = nz;
  double best = -1.0;
  // Items are (chunk, tile) pairs taken in rounds of `resident`; a round
  // costs the planes of its longest item plus `overhead` planes of start-up.
  for (int chunks = 1; chunks <= nz; ++chunks) {
    const int len = (nz + chunks - 1) / chunks;
    const int real_chunks = (nz + len - 1) / len;
    if (real_chunks != chunks) continue;  // same length as a smaller count
    const long long items = (long long)tiles * chunks;
    const long long rounds = (items + resident - 1) / resident;
    const double useful = (double)tiles * nz;
    const double cost = (double)rounds * resident * (len + overhead);
    const double eff = useful / cost;
    // prefer longer chunks when efficiency ties (fewer halo planes)
    if (eff > best + 1e-9) {
      best = eff;
      best_len = len;
    }
    if (len <= 4) break;
  }
  return best_len;
}

}  // namespace psg
