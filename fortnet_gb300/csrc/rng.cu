// Host-side parameter initialisation of the reference, so that training started here draws the
// same initial weights as the reference program for the same RandomSeed:
//  * RANLUX (luxury level 3) — the subtract-with-borrow generator of Marsaglia and Zaman with
//    Luescher's decimation (M. Luescher, Comput. Phys. Commun. 79 (1994) 100; F. James, ibid.
//    111), as used by lib_dftbp/ranlux.F90;
//  * normalXavier2d (lib_common/random.F90:122-181), drawn in TBpnn_init order
//    (lib_nn/bpnn.F90:133-136 -> network.F90:110-120 -> layer.F90:72-86);
//  * knuthShuffle (lib_common/random.F90:33-55).
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/fnetg.h"

namespace {

class Ranlux {
 public:
  Ranlux(int luxlev, int seed) {
    static const int skips[5] = {0, 24, 73, 199, 365};
    lux_ = (luxlev >= 0 && luxlev <= 4) ? luxlev : 3;
    skip_ = skips[lux_];
    long js = seed > 0 ? seed : 314159265;
    two_m24_ = 1.0;
    for (int k = 0; k < 24; k++) {
      two_m24_ *= 0.5;
      const long q = js / 53668;
      js = 40014 * (js - q * 53668) - q * 12211;
      if (js < 0) js += 2147483563;
      seed_[k] = (int)(js % (1 << 24));
    }
    two_m12_ = two_m24_ * 4096.0;
    i_ = 23;  // 0-based positions of the two lags
    j_ = 9;
    carry_ = (seed_[23] & ~((1 << 24) - 1)) ? 1 : 0;
    count_ = 0;
  }

  double next() {
    int v = step();
    double u = (double)v * two_m24_;
    if (u < two_m12_) {
      u += ((double)seed_[j_] * two_m24_) * two_m24_;
      if (u <= 0.0) u = two_m24_ * two_m24_;
    }
    if (++count_ == 24) {
      count_ = 0;
      for (int k = 0; k < skip_; k++) step();
    }
    return u;
  }

 private:
  int step() {
    int v = seed_[j_] - seed_[i_] - carry_;
    if (v & ~((1 << 24) - 1)) {
      v &= (1 << 24) - 1;
      carry_ = 1;
    } else {
      carry_ = 0;
    }
    seed_[i_] = v;
    i_ = i_ == 0 ? 23 : i_ - 1;
    j_ = j_ == 0 ? 23 : j_ - 1;
    return v;
  }

  int seed_[24];
  int lux_, skip_, i_, j_, carry_, count_;
  double two_m24_, two_m12_;
};

constexpr double kPi = 3.14159265358979323846;

struct RngHandle {
  Ranlux r;
};

}  // namespace

extern "C" {

// A RANLUX stream (luxury level 3) seeded like the reference's Options{RandomSeed}.
void *fnetg_rng_create(int32_t seed) { return new RngHandle{Ranlux(3, seed)}; }
void fnetg_rng_destroy(void *h) { delete static_cast<RngHandle *>(h); }
int fnetg_rng_uniform(void *h, double *out, int64_t n) {
  if (!h || (n > 0 && !out)) return FNETG_E_INVALID;
  for (int64_t k = 0; k < n; k++) out[k] = static_cast<RngHandle *>(h)->r.next();
  return FNETG_OK;
}

int fnetg_rng_init_params(void *h, int32_t nspecies, int32_t nlayer, const int32_t *dims,
                          double *params) {
  if (!h || !dims || !params || nlayer < 2 || nspecies < 1) return FNETG_E_INVALID;
  Ranlux &r = static_cast<RngHandle *>(h)->r;
  const int64_t np = fnetg_nparams(nlayer, dims);
  std::vector<int64_t> woff(nlayer), boff(nlayer);
  int64_t ind = 0;
  for (int l = 0; l < nlayer; l++) {
    woff[l] = ind;
    ind += (int64_t)dims[l] * (l < nlayer - 1 ? dims[l + 1] : 1);
  }
  for (int l = 0; l < nlayer; l++) {
    boff[l] = ind;
    ind += dims[l];
  }
  for (int s = 0; s < nspecies; s++) {
    double *p = params + (int64_t)s * np;
    for (int l = 0; l < nlayer; l++) {
      const int ncur = dims[l];
      const int nnext = l < nlayer - 1 ? dims[l + 1] : 1;
      const int64_t cnt = (int64_t)ncur * nnext;
      const double var = 2.0 / (double)(nnext + ncur);
      const double bound = std::sqrt(-2.0 * var * std::log(0.1 * std::sqrt(2.0 * kPi * var)));
      for (int64_t k = 0; k < cnt; k++) {
        const double x = (r.next() - 0.5) * 2.0 * bound;
        p[woff[l] + k] = std::exp(-0.5 * (x * x) / var) / std::sqrt(2.0 * kPi * var);
      }
      for (int k = 0; k < ncur; k++) p[boff[l] + k] = 0.0;
    }
    for (int k = 0; k < dims[nlayer - 1]; k++) p[woff[nlayer - 1] + k] = 0.0;
  }
  return FNETG_OK;
}

int fnetg_rng_shuffle(void *h, int32_t *arr, int32_t n) {
  if (!h || (n > 0 && !arr)) return FNETG_E_INVALID;
  Ranlux &r = static_cast<RngHandle *>(h)->r;
  for (int ii = n; ii >= 2; ii--) {
    const int pos = (int)(r.next() * ii);
    const int32_t t = arr[pos];
    arr[pos] = arr[ii - 1];
    arr[ii - 1] = t;
  }
  return FNETG_OK;
}

}  // extern "C"
