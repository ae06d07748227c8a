"""Mie series for the field inside a homogeneous sphere under a plane wave
(Bohren & Huffman, Absorption and Scattering of Light by Small Particles,
ch. 4: internal-field coefficients c_n, d_n and the vector spherical
harmonics M_o1n, N_e1n with spherical Bessel functions of the first kind).
A known answer for the tests of the VIE operator; not part of the library.
Convention exp(-i w t), incident E = x exp(i k z); conjugate for MARIE's
exp(+j w t), E = x exp(-j k z)."""
import numpy as np
from scipy.special import spherical_jn, spherical_yn


def mie_internal(points, a, k, m, nmax=None):
    """E (len(points), 3) inside a sphere of radius a centred at the origin,
    relative refractive index m, free-space wavenumber k, for the incident
    E = x exp(i k z); nmax terms (Wiscombe's rule by default)."""
    x = k * a
    if nmax is None:
        nmax = int(x + 4 * x ** (1 / 3) + 10)
    mx = m * x
    r = np.linalg.norm(points, axis=1)
    th = np.arccos(np.clip(points[:, 2] / r, -1, 1))
    ph = np.arctan2(points[:, 1], points[:, 0])
    mu = np.cos(th)
    rho = m * k * r
    E = np.zeros((len(r), 3), complex)
    pi_prev, pi_cur = np.zeros_like(mu), np.ones_like(mu)
    for n in range(1, nmax + 1):
        if n > 1:
            pi_new = ((2*n-1)/(n-1)) * mu * pi_cur - (n/(n-1)) * pi_prev
            pi_prev, pi_cur = pi_cur, pi_new
        tau = n * mu * pi_cur - (n + 1) * pi_prev
        jn, jnp = spherical_jn(n, x), spherical_jn(n, x, derivative=True)
        yn, ynp = spherical_yn(n, x), spherical_yn(n, x, derivative=True)
        hn, hnp = jn + 1j * yn, jnp + 1j * ynp
        xh_p = hn + x*hnp            # [x h_n(x)]'
        xj_p = jn + x*jnp
        jm, jmp = spherical_jn(n, mx), spherical_jn(n, mx, derivative=True)
        mxj_p = jm + mx*jmp          # [mx j_n(mx)]'
        cn = (jn*xh_p - hn*xj_p) / (jm*xh_p - hn*mxj_p)
        dn = (m*jn*xh_p - m*hn*xj_p) / (m**2*jm*xh_p - hn*mxj_p)
        En = 1j**n * (2*n+1) / (n*(n+1))
        z, zp = spherical_jn(n, rho), spherical_jn(n, rho, derivative=True)
        rz_p = z + rho*zp            # [rho z_n]'
        # M_o1n and N_e1n (spherical components r, theta, phi)
        M = np.stack([np.zeros_like(z), np.cos(ph)*pi_cur*z, -np.sin(ph)*tau*z], axis=1)
        N = np.stack([n*(n+1)*np.cos(ph)*np.sin(th)*pi_cur*z/rho, np.cos(ph)*tau*rz_p/rho, -np.sin(ph)*pi_cur*rz_p/rho], axis=1)
        E += En * (cn*M - 1j*dn*N)
    # spherical -> cartesian
    st, ct, sp, cp = np.sin(th), np.cos(th), np.sin(ph), np.cos(ph)
    Ex = E[:,0]*st*cp + E[:,1]*ct*cp - E[:,2]*sp
    Ey = E[:,0]*st*sp + E[:,1]*ct*sp + E[:,2]*cp
    Ez = E[:,0]*ct - E[:,1]*st
    return np.stack([Ex, Ey, Ez], axis=1)

