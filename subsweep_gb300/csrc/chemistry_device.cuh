// Hydrogen-only chemistry on the device: the semi-implicit x_HII / temperature
// update of Rosdahl et al. (2015) with recursive timestep halving, as in
// src/chemistry/hydrogen_only/mod.rs:125-461 of the reference.
//
// The reference recurses (perform_timestep_internal, 394-424): a failed attempt
// over dt is replaced by two attempts over dt/2, depth <= 100.  Here the recursion
// is an explicit loop.  At any time at most one second half is pending per depth,
// and pending halves are taken deepest first, so the pending set is a bitmask
// over depths and the next interval is its highest set bit.  The result (state and
// the timescale of the last accepted substep) is the same as the recursion's.
//
// kCarryNeutral = false restates the reference exactly: the neutral fraction is
// recomputed as (1 - x) wherever it is used.  kCarryNeutral = true (mixed path)
// additionally carries y = 1 - x as its own FP64 state, updated by -dx, so the
// neutral density keeps full relative precision near complete ionisation; the
// smaller of x and y is the accurate one and the other is re-derived from it.
//
// Work per try_timestep_update attempt: the FP64 path (the reference's expressions) 535
// DFMA, 128 DADD and 169 DMUL thread instructions, 1367 FP64 flops (ncu, C2 64^3).  The
// mixed path evaluates the rate fits in FP32 (Fits32), forms the per-cell factors once
// per cell, and keeps the densities, the sums, the implicit updates and their accept /
// reject tests in FP64: 55 DFMA, 41 DMUL and 9 DADD, 160 FP64 flops (ncu, C4 64^3).
#pragma once

#include <cfloat>
#include <cstdint>

namespace swk {

// src/units/mod.rs:14-108, every quantity a plain SI double.
struct Units {
  static constexpr double kCentimeters = 0.01;
  static constexpr double kCentimetersSquared = kCentimeters * kCentimeters;
  static constexpr double kCubicCentimeters = 1e-6;
  static constexpr double kSeconds = 1.0;
  static constexpr double kCentimetersCubedPerS = kCubicCentimeters / kSeconds;
  static constexpr double kErgs = 1e-7;
  static constexpr double kErgsCentimetersCubedPerS = kErgs * kCentimetersCubedPerS;
  static constexpr double kErgsPerS = kErgs / kSeconds;
  static constexpr double kElectronVolts = 1.602176634e-19;
  static constexpr double kBoltzmann = 1.380649e-23;
  static constexpr double kProtonMass = 1.67262192369e-27;
  static constexpr double kGamma = 5.0 / 3.0;
  static constexpr double kSigma = 2.9580524545305314e-18 * kCentimetersSquared;
  static constexpr double kPhotonAverageEnergy = 18.028356312818811 * kElectronVolts;
  static constexpr double kRydberg = 13.65693 * kElectronVolts;
};

constexpr int kChemMaxDepth = 100;               // hydrogen_only/mod.rs:34
constexpr double kIonizedFractionEpsilon = 1e-10;  // hydrogen_only/mod.rs:38

enum ChemProcess : int { kProcTemperature = 0, kProcIonization = 1, kProcPhotonRate = 2 };

struct Timescale {
  double time;
  int process;
};

// chemistry/timescale.rs:114-120: strict <, so NaN selects `b`.
__device__ __forceinline__ Timescale ts_min(Timescale a, Timescale b) {
  return a.time < b.time ? a : b;
}

// Mixed path: the Rosdahl et al. (2015) rate fits and their temperature derivatives
// (hydrogen_only/mod.rs:161-273) evaluated in FP32 in the fits' own units (erg cm^3/s,
// cm^3/s), at one temperature: the shared factors as in the FP64 forms below (one
// reciprocal of T, rsqrt for both square roots, exp / log1p for the powers).  The
// values carry ~1e-6 relative error; they enter the FP64 update as coefficients.
struct Fits32 {
  float fit, fitd;          // collision_fit and its derivative (161-173)
  float exc, dexc;          // collisional excitation cooling / 7.5e-19-scaled form, and d/dT (237-253)
  float recc, drecc;        // case B recombination cooling and d/dT (196-216)
  float brems, dbrems;      // bremsstrahlung cooling and d/dT (255-263)
  float alpha, dalpha;      // case B recombination rate and d/dT (175-194)
};

__device__ __forceinline__ Fits32 fits32(float t) {
  Fits32 f;
  const float inv_t = 1.0f / t;
  const float rsq = rsqrtf(t);
  const float sq = t * rsq;                      // sqrt(t)
  const float s5 = sq * 0.0031622777f;           // sqrt(t / 1e5)
  const float inv_s5 = rsq * 316.22776f;         // 1 / sqrt(t / 1e5)
  const float inv_1s5 = 1.0f / (1.0f + s5);
  // collision fit
  const float c1 = 1e-5f, c2 = 157809.1f;
  const float e = expf(-c2 * inv_t);
  f.fit = sq * inv_1s5 * e;
  f.fitd = (e * (c1 * c2 * t + 0.5f * s5 * (2.0f * c2 + t))) * (inv_t * rsq) * inv_s5 * (inv_1s5 * inv_1s5);
  // collisional excitation cooling
  const float c2e = 118348.0f;
  const float e_exc = expf(-c2e * inv_t);
  f.exc = 7.5e-19f * inv_1s5 * e_exc;
  f.dexc = (7.5e-19f * e_exc * (c2e * c1 * t - 0.5f * c1 * (t * t) + c2e * s5)) * (inv_t * inv_t) * inv_s5 *
           (inv_1s5 * inv_1s5);
  // case B recombination cooling: lambda^1.97 and (lambda / 2.25)^0.376 from one logarithm
  const float lambda = 315614.0f * inv_t;
  const float ln_lambda = logf(lambda);
  const float l197 = expf(1.97f * ln_lambda);
  const float q = expf(0.376f * (ln_lambda - 0.81093021f));  // ln 2.25
  const float inv_a = expf(-3.72f * log1pf(q));               // (1 + q)^-3.72
  f.recc = 3.435e-30f * t * l197 * inv_a;
  f.drecc = 3.435e-30f * ((inv_a / (1.0f + q)) * (1.0f - 1.97f + (1.0f - 1.97f + 0.376f * 3.72f) * q) * l197);
  // bremsstrahlung
  f.brems = 1.42e-27f * sq;
  f.dbrems = 1.42e-27f * 0.5f * rsq;
  // case B recombination rate: (lambda / 2.74)^0.407, (1 + p)^-2.242
  const float sl = 561.79534f * rsq;                          // sqrt(lambda)
  const float p = expf(0.407f * (ln_lambda - 1.0079579f));    // ln 2.74
  const float inv_b = expf(-2.242f * log1pf(p));
  f.alpha = 2.753e-14f * (lambda * sl) * inv_b;
  const float da = -sl * (inv_b / (p + 1.0f)) * (0.407f * 2.242f * p - 1.5f * p - 1.5f);
  f.dalpha = (2.753e-14f * da) * (-lambda * inv_t);  // d lambda / dT = -lambda / T
  return f;
}

template <bool kCarryNeutral>
struct ChemSolver {
  double x;   // ionized hydrogen fraction
  double y;   // neutral fraction (only meaningful when kCarryNeutral)
  double temperature;
  double density, volume, length, rate, scale_factor;
  bool has_floor;
  double floor_t, floor_x;
  bool clamp_invalid;
  // Mixed path: the per-cell factors of the update, formed once per cell instead of once
  // per attempt (prepare(); the FP64 path keeps the reference's expressions)
  double nh_cell, k_cell, rate_per_volume, compton_cell, xx_cell;

  __device__ void prepare() {
    if (!kCarryNeutral) return;
    nh_cell = density / Units::kProtonMass;
    k_cell = (Units::kGamma - 1.0) * Units::kProtonMass / (density * Units::kBoltzmann);
    rate_per_volume = rate / volume;
    xx_cell = 2.727 / scale_factor;
    const double x2 = xx_cell * xx_cell;
    compton_cell = (1.017e-37 * (x2 * x2)) * Units::kErgsPerS;
  }

  __device__ __forceinline__ double neutral() const { return kCarryNeutral ? y : (1.0 - x); }
  __device__ __forceinline__ double nh() const {
    return kCarryNeutral ? nh_cell : density / Units::kProtonMass;
  }
  __device__ __forceinline__ double n_ionized() const { return nh() * x; }
  __device__ __forceinline__ double n_neutral() const { return nh() * neutral(); }
  __device__ __forceinline__ double mu() const { return 1.0 / (x + 1.0); }

  // The rate fits and their temperature derivatives (161-302) share their powers and
  // exponentials: each derivative below is the reference's formula with the common
  // factor taken from the fit evaluated at the same temperature
  // ((1 + p)^(-c - 1) = 1 / ((1 + p)^c (1 + p)), lambda^1.5 = lambda sqrt(lambda)).
  // The values agree with separate evaluation to rounding.

  // collision_fit 161-166 and collision_fit_derivative 167-173
  __device__ static void collision_fits(double t, double sqrt_t, double s5, double& fit, double& fitd) {
    const double c1 = 1.0 / 1e5, c2 = 157809.1;
    const double e = exp(-c2 / t);
    fit = sqrt_t / (1.0 + s5) * e;
    fitd = (e * (c1 * c2 * t + 0.5 * s5 * (2.0 * c2 + t))) / ((t * sqrt_t) * s5 * ((s5 + 1.0) * (s5 + 1.0)));
  }

  // Mixed path: cooling_rate and its derivative from the FP32 fits; the densities, the
  // sums and the unit factors in FP64.
  __device__ void cooling32(double& lambda_c, double& dlambda_c) const {
    const double t = temperature;
    const double ne = n_ionized();
    const double nhn = n_neutral();
    const double nhi = n_ionized();
    const Fits32 f = fits32((float)t);
    const double u = Units::kErgsCentimetersCubedPerS;
    const double compton = compton_cell * (t - xx_cell);
    const double dcompton = compton_cell;
    const double coll = ((double)f.exc + 1.27e-21 * (double)f.fit) * u * ne * nhn;
    const double dcoll = ((double)f.dexc + 1.27e-21 * (double)f.fitd) * u * ne * nhn;
    lambda_c = coll + ((double)f.recc + (double)f.brems) * u * ne * nhi + compton * ne;
    dlambda_c = dcoll + ((double)f.drecc + (double)f.dbrems) * u * ne * nhi + dcompton * ne;
  }

  // cooling_rate 275-287 and cooling_rate_derivative 289-302 at the current temperature:
  // collisional ionization / excitation cooling (237-253), case B recombination cooling
  // (196-216), bremsstrahlung and Compton cooling (265-273).
  __device__ void cooling(double& lambda_c, double& dlambda_c) const {
    const double t = temperature;
    const double ne = n_ionized();
    const double nhn = n_neutral();
    const double nhi = n_ionized();
    const double sq = sqrt(t);
    const double s5 = sqrt(t / 1e5);
    double fit, fitd;
    collision_fits(t, sq, s5, fit, fitd);
    // excitation cooling and its derivative
    const double e_exc = exp(-118348.0 / t);
    const double exc = (7.5e-19 / (1.0 + s5) * e_exc) * Units::kErgsCentimetersCubedPerS;
    const double c3 = 1.0 / 1e5, c2e = 118348.0;
    const double dexc = ((7.5e-19 * e_exc * (c2e * c3 * t - 0.5 * c3 * (t * t) + c2e * s5)) /
                         ((t * t) * s5 * ((1.0 + s5) * (1.0 + s5)))) *
                        Units::kErgsCentimetersCubedPerS;
    // case B recombination cooling and its derivative
    const double lambda = 315614.0 / t;
    // lambda^1.97 and (lambda / 2.25)^0.376 from one logarithm
    const double ln_lambda = log(lambda);
    const double l197 = exp(1.97 * ln_lambda);
    const double q = exp(0.376 * (ln_lambda - 0.81093021621632877));  // ln 2.25
    const double a = pow(1.0 + q, 3.72);
    const double recomb_rate = (3.435e-30 * t * l197 / a) * Units::kErgsCentimetersCubedPerS;
    const double c2r = 1.97, c3r = 0.376, c4r = 3.72;
    const double drecomb_rate = (3.435e-30 * ((1.0 / (a * (1.0 + q))) *
                                             (1.0 - 1.0 * c2r + (1.0 - 1.0 * c2r + c3r * c4r) * q) * l197)) *
                                Units::kErgsCentimetersCubedPerS;
    // Compton
    const double xx = 2.727 / scale_factor;
    const double x2 = xx * xx;
    const double compton = (1.017e-37 * (x2 * x2) * (t - xx)) * Units::kErgsPerS;
    const double dcompton = (1.017e-37 * (x2 * x2)) * Units::kErgsPerS;

    const double coll = (exc + (1.27e-21 * fit) * Units::kErgsCentimetersCubedPerS) * ne * nhn;
    const double recomb = recomb_rate * ne * nhi;
    const double brems = ((1.42e-27 * sq) * Units::kErgsCentimetersCubedPerS) * ne * nhi;
    lambda_c = coll + recomb + brems + compton * ne;
    const double dcoll = (dexc + (1.27e-21 * fitd) * Units::kErgsCentimetersCubedPerS) * ne * nhn;
    const double drecomb = drecomb_rate * ne * nhi;
    const double dbrems = ((1.42e-27 / (2.0 * sq)) * Units::kErgsCentimetersCubedPerS) * ne * nhi;
    dlambda_c = dcoll + drecomb + dbrems + dcompton * ne;
  }

  // 312-319: photons absorbed per photon arriving, 1 - exp(-n_HI sigma size); both
  // updates of an attempt use it with the x of the attempt's start.  Mixed path:
  // -expm1 in FP32, accurate to ~1e-7 relative also for optically thin cells.
  __device__ double absorbed_fraction() const {
    if (kCarryNeutral) return -(double)expm1f((float)(-n_neutral() * Units::kSigma * length));
    return 1.0 - exp(-n_neutral() * Units::kSigma * length);
  }

  // 304-310 (+ photoheating_rate 321-325); m = mu() of the attempt
  __device__ double temperature_change(double timestep, double absorbed, double m) const {
    double k, heating, lc, dlc;
    if (kCarryNeutral) {
      k = k_cell;
      heating = (rate_per_volume * absorbed) * (Units::kPhotonAverageEnergy - Units::kRydberg);
      cooling32(lc, dlc);
    } else {
      k = (Units::kGamma - 1.0) * Units::kProtonMass / (density * Units::kBoltzmann);
      heating = ((timestep * rate * absorbed) / volume) * (Units::kPhotonAverageEnergy - Units::kRydberg) / timestep;
      cooling(lc, dlc);
    }
    double lambda = heating - lc;
    double dlambdadt = -dlc;
    return k * m * lambda * timestep / (1.0 - k * m * dlambdadt * timestep);
  }
  // 334-354 (+ photoionization_rate 327-332), case B rate 175-194 at the current
  // (already updated) temperature
  __device__ double ionized_fraction_change(double timestep, double absorbed, double m) const {
    const double t = temperature;
    double n_h = nh();
    double ne = n_ionized();
    double alpha, dalpha, fit, fitd, photo;
    const double c2a = 0.407, c3a = 2.242;
    if (kCarryNeutral) {
      const Fits32 f = fits32((float)t);
      alpha = (double)f.alpha * Units::kCentimetersCubedPerS;
      dalpha = (double)f.dalpha * Units::kCentimetersCubedPerS;
      fit = (double)f.fit;
      fitd = (double)f.fitd;
      photo = (rate_per_volume * absorbed) / n_neutral();
    } else {
      const double lambda = 315614.0 / t;
      const double dlambda_dt = -315614.0 / (t * t);
      const double sl = sqrt(lambda);
      const double p = pow(lambda / 2.74, 0.407);
      const double b = pow(1.0 + p, 2.242);
      alpha = (2.753e-14 * (lambda * sl) / b) * Units::kCentimetersCubedPerS;
      const double da = -sl * (1.0 / (b * (p + 1.0))) * (c2a * c3a * p - 1.5 * p - 1.5);
      dalpha = ((2.753e-14 * da) * Units::kCentimetersCubedPerS) * dlambda_dt;
      const double sq = sqrt(t);
      const double s5 = sqrt(t / 1e5);
      collision_fits(t, sq, s5, fit, fitd);
      photo = (((timestep * rate) * absorbed) / (n_neutral() * volume)) / timestep;
    }
    double beta = (5.85e-11 * fit) * Units::kCentimetersCubedPerS;
    double dbeta = (5.85e-11 * fitd) * Units::kCentimetersCubedPerS;
    double c = beta * ne + photo;
    double d = alpha * ne;
    double xhii = x;
    double rhsc = ne * t * m * 1.0 * dbeta;
    double dcdx = n_h * beta - rhsc;
    double rhsd = ne * t * m * 1.0 * dalpha;
    double dddx = n_h * alpha - rhsd;
    double j = dcdx - (c + d) - xhii * (dcdx + dddx);
    return timestep * (c - xhii * (c + d)) / (1.0 - j * timestep);
  }

  // 356-369 with Rust f64::clamp semantics (asserts min <= max: flagged here).
  __device__ void clamp() {
    double xf = has_floor ? floor_x : kIonizedFractionEpsilon;
    const double xmax = 1.0 - kIonizedFractionEpsilon;
    if (!(xf <= xmax)) clamp_invalid = true;
    if (kCarryNeutral) {
      if (x < xf) { x = xf; y = 1.0 - x; }
      if (x > xmax) { x = xmax; y = kIonizedFractionEpsilon; }
    } else {
      if (x < xf) x = xf;
      if (x > xmax) x = xmax;
    }
    if (has_floor && temperature < floor_t) temperature = floor_t;
  }

  // update() 444-461
  __device__ __forceinline__ static bool accept(double value, double change, double max_allowed,
                                                double timestep, double& recommendation) {
    double relative_change = fmin(fabs(change / value), 1.0 / DBL_EPSILON);
    if (relative_change > max_allowed) return false;
    recommendation = timestep * (max_allowed / relative_change);
    return true;
  }

  // try_timestep_update 371-392
  __device__ bool try_update(double timestep, double safety, Timescale& out) {
    const double absorbed = absorbed_fraction();
    const double m = mu();  // both updates use the x of the attempt's start
    double tc = temperature_change(timestep, absorbed, m);
    double rec_t;
    if (!accept(temperature, tc, safety, timestep, rec_t)) return false;
    temperature += tc;
    double xc = ionized_fraction_change(timestep, absorbed, m);
    double rec_x;
    if (!accept(x, xc, safety, timestep, rec_x)) return false;
    x += xc;
    if (kCarryNeutral) {
      y -= xc;
      // keep the smaller fraction exact and derive the other from it
      if (x < 0.5) y = 1.0 - x; else x = 1.0 - y;
    }
    clamp();
    out = ts_min(Timescale{rec_t, kProcTemperature}, Timescale{rec_x, kProcIonization});
    return true;
  }

  // perform_timestep 426-441 with perform_timestep_internal 394-424 unrolled.
  __device__ Timescale perform_timestep(double timestep, double safety, bool& failed,
                                        uint32_t& attempts) {
    uint64_t pend_lo = 0, pend_hi = 0;  // pending second halves at depths 1..127
    int depth = 0;
    Timescale last{0.0, kProcTemperature};
    while (true) {
      clamp();
      double t0 = temperature, x0 = x, y0 = y;
      if (depth > kChemMaxDepth) {
        failed = true;
        return Timescale{timestep / 10.0, kProcTemperature};
      }
      double sub = ldexp(timestep, -depth);  // == timestep / 2^depth, exact
      ++attempts;
      Timescale r;
      if (!try_update(sub, safety, r)) {
        temperature = t0;
        x = x0;
        y = y0;
        ++depth;
        if (depth < 64) pend_lo |= (1ull << depth); else pend_hi |= (1ull << (depth - 64));
        continue;
      }
      last = r;
      if (pend_hi) {
        depth = 127 - __clzll((long long)pend_hi);
        pend_hi &= ~(1ull << (depth - 64));
      } else if (pend_lo) {
        depth = 63 - __clzll((long long)pend_lo);
        pend_lo &= ~(1ull << depth);
      } else {
        failed = false;
        return last;
      }
    }
  }
};

}  // namespace swk
