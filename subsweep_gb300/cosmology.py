"""The cosmology the input path needs (src/cosmology.rs): the scale factor a and little h
that convert Arepo's comoving units, and, for stellar ages, the cosmic time between two
scale factors in a flat Lambda-CDM universe."""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

HUBBLE = 3.2407789e-18  # H0 / h in 1/s (src/cosmology.rs:86)
YEAR = 3.15576e7         # s (src/units/mod.rs:48)


@dataclasses.dataclass(frozen=True)
class Cosmology:
    """Cosmology::Cosmological {a, h, params} (src/cosmology.rs:14-29); `omega_0` and
    `omega_lambda` are CosmologyParams, needed only for times between scale factors."""
    a: float
    h: float
    omega_0: Optional[float] = None
    omega_lambda: Optional[float] = None

    def factor(self, d) -> float:
        """Cosmology::get_factor (src/cosmology.rs:56-61) of a unit with exponents d.a and
        d.h: a^(-d.a) * h^(-d.h)."""
        return float(self.a) ** (-d.a) * float(self.h) ** (-d.h)

    def _time(self, a: float) -> float:
        ol, o0 = self.omega_lambda, self.omega_0
        factor1 = 2.0 / (3.0 * math.sqrt(ol))
        term1 = math.sqrt(ol / o0) * a ** 1.5
        term2 = math.sqrt(1.0 + ol / o0 * (a * a * a))
        return factor1 * math.log(term1 + term2)

    def time_difference_between_scalefactors(self, a0: float, a1: float) -> float:
        """Seconds from scale factor a0 to a1 (CosmologyParams::
        time_difference_between_scalefactors, src/cosmology.rs:80-104): the flat
        Lambda-CDM age 2 / (3 sqrt(O_L)) ln(sqrt(O_L / O_0) a^1.5 + sqrt(1 + O_L / O_0 a^3))
        in units of 1 / H0."""
        if self.omega_0 is None or self.omega_lambda is None:
            raise ValueError("Tried to compute time difference in non cosmological run "
                             "(omega_0 and omega_lambda are needed)")
        if abs((self.omega_lambda + self.omega_0) - 1.0) > 1e-2:
            raise NotImplementedError("Cosmology needs to be flat.")
        return (self._time(a1) - self._time(a0)) / (HUBBLE * self.h)

    def scalefactor_after(self, a: float, delta_t: float) -> float:
        """The scale factor delta_t seconds after scale factor a
        (get_scalefactor_from_scalefactor_and_time_difference, src/cosmology.rs:108-125):
        bisection on [0, 1] until the time difference is within 100 years of delta_t, at
        most 101 halvings."""
        lo, hi = 0.0, 1.0
        threshold = 100.0 * YEAR
        for _ in range(101):
            guess = (lo + hi) / 2.0
            val = self.time_difference_between_scalefactors(a, guess) - delta_t
            if abs(val) <= threshold:
                return guess
            if math.copysign(1.0, val) < 0:
                lo = guess
            else:
                hi = guess
        raise ValueError("Binary search failed")
