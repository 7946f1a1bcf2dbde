"""Exact internal energy of the finite 2D Ising model on an m x n torus.

Kaufman's partition function (B. Kaufman, Phys. Rev. 76, 1232 (1949), in the
form of Ferdinand & Fisher, Phys. Rev. 185, 832 (1969), eqs. 2.1-2.3):

    Z = 1/2 (2 sinh 2K)^(mn/2) (Z1 + Z2 + Z3 + Z4),
    Z1 = prod_r 2 cosh(m g_{2r+1} / 2),  Z2 = prod_r 2 sinh(m g_{2r+1} / 2),
    Z3 = prod_r 2 cosh(m g_{2r} / 2),    Z4 = prod_r 2 sinh(m g_{2r} / 2),
    cosh g_l = cosh 2K coth 2K - cos(pi l / n)  (r = 0 .. n-1),
    g_0 = 2K + ln tanh K  (negative below T_c),

with K = J / T.  The energy per spin in bond counting (the reference's
Exchange::total_energy, src/energy.rs:208-213) is u = -(1/mn) d ln Z / dK,
taken here by a central difference in 50-digit arithmetic.  An axis of
extent 2 counts its bond twice, as the lattices of this library do.
Checked against brute-force enumeration of small tori in tests/test_oracle.py.
"""
import mpmath as mp


def log_partition(K, m, n, dps=50):
    with mp.workdps(dps):
        K = mp.mpf(K)
        c = mp.cosh(2 * K) / mp.tanh(2 * K)

        def gamma(l):
            if l == 0:
                return 2 * K + mp.log(mp.tanh(K))
            return mp.acosh(c - mp.cos(mp.pi * l / n))

        z1 = z2 = z3 = z4 = mp.mpf(1)
        for r in range(n):
            g1, g0 = gamma(2 * r + 1), gamma(2 * r)
            z1 *= 2 * mp.cosh(m * g1 / 2)
            z2 *= 2 * mp.sinh(m * g1 / 2)
            z3 *= 2 * mp.cosh(m * g0 / 2)
            z4 *= 2 * mp.sinh(m * g0 / 2)
        return mp.log(mp.mpf(1) / 2 * (2 * mp.sinh(2 * K)) ** (mp.mpf(m * n) / 2) * (z1 + z2 + z3 + z4))


def energy_per_spin(T, m, n, J=1.0):
    """Exact <E>/N in bond counting, E = -J sum_bonds s_i s_j, on an m x n torus."""
    with mp.workdps(60):
        K = mp.mpf(J) / mp.mpf(T)
        h = mp.mpf("1e-15")
        d = (log_partition(K + h, m, n, 60) - log_partition(K - h, m, n, 60)) / (2 * h)
        return float(-J * d / (m * n))
