"""Seeded synthetic data: splitmix64 streams and random Fourier-mode fields.

The coefficient field has the form of ugcore's LognormalRandomField::eval_K
(lib_disc/spatial_disc/user_data/common_user_data/lognormal_random_field_impl.h):
g(x) = sqrt(2/N) * sum_m cos(k_m . x + phase_m), K = exp(factor * g).  The
reference draws its modes with rand(); here a counter-based splitmix64 stream
makes every mode reproducible on any machine.  The velocity field is the curl
of a random vector potential A(x) = sum_m a_m cos(k_m . x + phase_m):
v(x) = scale * sum_m -sin(k_m . x + phase_m) (k_m x a_m).
Wave vectors are 2*pi*kappa with kappa uniform in the ball |kappa| <= kmax.
"""
import math

import numpy as np

MASK = (1 << 64) - 1
TWO_PI = 6.283185307179586


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014)."""

    def __init__(self, seed):
        self.state = seed & MASK

    def next(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self):
        return float(self.next() >> 11) * (1.0 / 9007199254740992.0)

    def gauss(self):
        u1 = 1.0 - self.uniform()
        u2 = self.uniform()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(TWO_PI * u2)

    def wavevector(self, dim, kmax):
        while True:
            kap = [0.0, 0.0, 0.0]
            r2 = 0.0
            for d in range(dim):
                kap[d] = kmax * (2.0 * self.uniform() - 1.0)
                r2 += kap[d] * kap[d]
            if r2 <= kmax * kmax and r2 > 0.0:
                return [TWO_PI * kap[d] for d in range(dim)]


def hash_uniform(seed, i):
    """U[0,1) from the pair (seed, i): one splitmix64 step of seed ^ (i*C)."""
    s = SplitMix64((seed ^ ((i * 0xD1B54A32D192ED03) & MASK)) & MASK)
    return float(s.next() >> 11) * (1.0 / 9007199254740992.0)


def source_uniform(seed, n):
    return np.array([2.0 * hash_uniform(seed, i) - 1.0 for i in range(n)])


class ScalarField:
    """g(x) = amp * sum_m cos(k_m . x + phase_m), amp = sqrt(2/N)."""

    def __init__(self, dim, nmodes, kmax, seed):
        st = SplitMix64(seed)
        self.dim, self.nmodes = dim, nmodes
        self.amp = math.sqrt(2.0 / nmodes)
        k, ph = [], []
        for _ in range(nmodes):
            k.append(st.wavevector(dim, kmax))
            ph.append(TWO_PI * st.uniform())
        self.k = np.array(k, dtype=np.float64).reshape(nmodes, dim)
        self.phase = np.array(ph, dtype=np.float64)

    def __call__(self, x):
        x = np.atleast_2d(x)
        return self.amp * np.cos(x @ self.k.T + self.phase).sum(axis=1)


class CurlField:
    """v(x) = scale * sum_m -sin(k_m . x + phase_m) c_m, c_m = k_m x a_m, scaled so |v| <= 1."""

    def __init__(self, nmodes, kmax, seed):
        st = SplitMix64(seed)
        self.nmodes = nmodes
        k, ph, c = [], [], []
        bound = 0.0
        for _ in range(nmodes):
            km = st.wavevector(3, kmax)
            ph.append(TWO_PI * st.uniform())
            a = [st.gauss() for _ in range(3)]
            cm = [km[1] * a[2] - km[2] * a[1], km[2] * a[0] - km[0] * a[2], km[0] * a[1] - km[1] * a[0]]
            bound += math.sqrt(cm[0] * cm[0] + cm[1] * cm[1] + cm[2] * cm[2])
            k.append(km)
            c.append(cm)
        self.k = np.array(k, dtype=np.float64)
        self.c = np.array(c, dtype=np.float64)
        self.phase = np.array(ph, dtype=np.float64)
        self.scale = 1.0 / bound if bound > 0.0 else 1.0

    def __call__(self, x):
        x = np.atleast_2d(x)
        s = -np.sin(x @ self.k.T + self.phase)
        return self.scale * (s @ self.c)


# seed offsets shared with the oracle (oracle/ug4_oracle_api.c)
COEF_SEED_XOR = 0xC0EF
VEL_SEED_XOR = 0x7E10C17
