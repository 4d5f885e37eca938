// Strain rate from the non-equilibrium second-order moments of one node.
//
// Restates the moment-space method of the reference's sijstat01
// (Channel-Flow/saveload.f90:2322-2379, after Yu et al., Computers & Fluids 35,
// 957-965, 2006, Appendix): with the non-equilibrium parts of the energy
// moment e and of 3p_xx, p_ww, p_xy, p_yz, p_xz, each times the rate that
// relaxes it (s1 for e, s9 for the stress moments),
//   S_xx = -(n_e + 19 n_3pxx) / 38
//   S_yy = -(2 n_e - 19 (n_3pxx - 3 n_pww)) / 76
//   S_zz = -(2 n_e - 19 (n_3pxx + 3 n_pww)) / 76
//   S_xy = -1.5 n_pxy,  S_yz = -1.5 n_pyz,  S_zx = -1.5 n_pxz.
// The moments are written as sums over the lattice vectors (row weights
// -30/-11/8 by |c|^2 for e, 3c_x^2 - |c|^2 for 3p_xx, c_y^2 - c_z^2 for
// p_ww, c_a c_b for the off-diagonal ones), so the population numbering does
// not enter.  f: stored deviations f_i - w_i; rho, u: the macrovar values
// (deviation density, velocity including F/2).  Reference axes: x is the
// wall-normal direction.
#pragma once

namespace lbm {

template <typename R>
__host__ __device__ inline void strain_from_moments(const R f[Q], R rho, R ux, R uy, R uz, R s1, R s9, R S[6]) {
    R e = 0, p3 = 0, pw = 0, pxy = 0, pyz = 0, pxz = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const int cx = CXf(i), cy = CYf(i), cz = CZf(i);
        const int c2 = cx * cx + cy * cy + cz * cz;
        const R fi = f[i];
        e += (c2 == 0 ? R(-30) : (c2 == 1 ? R(-11) : R(8))) * fi;
        p3 += R(3 * cx * cx - c2) * fi;
        pw += R(cy * cy - cz * cz) * fi;
        if (cx * cy) pxy += R(cx * cy) * fi;
        if (cy * cz) pyz += R(cy * cz) * fi;
        if (cx * cz) pxz += R(cx * cz) * fi;
    }
    const R ux2 = ux * ux, uy2 = uy * uy, uz2 = uz * uz;
    const R ne = s1 * (e - (R(-11) * rho + R(19) * (ux2 + uy2 + uz2)));
    const R np = s9 * (p3 - (R(2) * ux2 - uy2 - uz2));
    const R nw = s9 * (pw - (uy2 - uz2));
    S[0] = -(ne + R(19) * np) / R(38);
    S[1] = -(R(2) * ne - R(19) * (np - R(3) * nw)) / R(76);
    S[2] = -(R(2) * ne - R(19) * (np + R(3) * nw)) / R(76);
    S[3] = R(-1.5) * s9 * (pxy - ux * uy);
    S[4] = R(-1.5) * s9 * (pyz - uy * uz);
    S[5] = R(-1.5) * s9 * (pxz - ux * uz);
}

}  // namespace lbm
