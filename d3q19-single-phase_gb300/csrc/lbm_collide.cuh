// D3Q19 MRT collision with split (Guo-type) forcing, one lattice node.
//
// Physics restated from the reference's collision_MRT
// (Channel-Flow/collision.f90:64-220, rates and coefficients para.f90:106-174):
//   Fbar_i = w_i (3 c_i.F + 9 (c_i.F)(c_i.u) - 3 u.F)           (:64-82)
//   f9     = f + Fbar/2                                         (:84)
//   m      = M f9,  m* = m - S (m - m_eq(rho, j))               (:86-154)
//   f*     = M^-1 m* + Fbar/2                                   (:157-220,:230)
// with M the orthogonal d'Humieres (2002) moment matrix, rho = sum f and
// j = sum c f + F/2 (macrovar, :398-418).
//
// GB300 formulation (same mathematics, fewer operations and better rounding):
// because M^-1 = M^T diag(1/|row_k|^2) and Fbar = M^-1 (M Fbar), the update is
// written as an increment of the stored populations,
//   f* = f + M^T diag(1/d) (MF - S (M f + MF/2 - m_eq)),   MF = M Fbar,
// where MF is known in closed form (it only has e, eps, j, q, p and pi
// components).  Moments and the back-transform use the opposite-pair
// sums/differences (even moments see f_i + f_opp, odd moments f_i - f_opp),
// about 210 floating-point operations per node.
//
// Populations are handled in scaled units g = S (f - w) (S = 1 except for FP16
// storage); the scale is folded into the constants: terms linear in F carry S,
// terms quadratic in the velocity use j_scaled * u_true.
#pragma once

namespace lbm {

template <typename R>
struct CollideConsts {
    R S, invS;              // storage scale and its inverse
    R Fx, Fy, Fz;           // body force, true units, reference axes
    R hFx, hFy, hFz;        // S F / 2: added to sum c f to give j
    R ajx, ajy, ajz;        // S F / 10: conserved-momentum increment / |row|^2
    R fqx, fqy, fqz;        // -(2/3) S F / 40: forcing part of the q increment
    R thFx, thFy, thFz;     // S F / 3: turns j into the q-equilibrium offset
    R ke, keps, kq, kp, kpi, kxy, km;  // s_k / |row_k|^2
    R kw, kwi;              // s9/12 and s10/24 (p_ww, pi_ww rows)
    R oeps, oepsj, oxx;     // omegepsl, omegepslj, omegxx
};

// Relax the populations f[0..18] of one node in place.
//   FROZEN = false : rho = sum f, j = sum c f + S F/2 (the normal step)
//   FROZEN = true  : rho = sum f, j = S * uf (velocity frozen, pre-relaxation)
//   YF = true      : the force has only a streamwise (reference y) component,
//                    as FORCING sets it (collision.f90:522-524); the terms with
//                    Fx or Fz are dropped instead of multiplied by zero
// rho_out / j_out receive the macroscopic values used (scaled units).
template <typename R, bool FROZEN, bool YF = false>
__device__ __forceinline__ void collide(R f[Q], const CollideConsts<R>& c,
                                        R ufx, R ufy, R ufz,
                                        R& rho_out, R& jx_out, R& jy_out, R& jz_out)
{
    // opposite-pair sums (even) and differences (odd)
    const R s1 = f[1] + f[2],   d1 = f[1] - f[2];
    const R s3 = f[3] + f[4],   d3 = f[3] - f[4];
    const R s5 = f[5] + f[6],   d5 = f[5] - f[6];
    const R s7 = f[7] + f[10],  d7 = f[7] - f[10];
    const R s8 = f[8] + f[9],   d8 = f[8] - f[9];
    const R s11 = f[11] + f[14], d11 = f[11] - f[14];
    const R s12 = f[12] + f[13], d12 = f[12] - f[13];
    const R s15 = f[15] + f[18], d15 = f[15] - f[18];
    const R s16 = f[16] + f[17], d16 = f[16] - f[17];

    const R syz5 = s3 + s5;              // y and z axis pairs
    const R sa = s1 + syz5;              // all axis populations
    const R sxy = s7 + s8, sxz = s11 + s12, syz = s15 + s16;
    const R sxyz = sxy + sxz;
    const R sd = sxyz + syz;             // all diagonal populations
    const R rho = f[0] + (sa + sd);

    const R Dx = (d7 - d8) + (d11 - d12);
    const R Dy = (d7 + d8) + (d15 - d16);
    const R Dz = (d11 + d12) + (d15 + d16);
    const R jfx = d1 + Dx, jfy = d3 + Dy, jfz = d5 + Dz;   // sum c f

    R jx, jy, jz;
    if (FROZEN) { jx = c.S * ufx; jy = c.S * ufy; jz = c.S * ufz; }
    else if (YF) { jx = jfx; jy = jfy + c.hFy; jz = jfz; }
    else        { jx = jfx + c.hFx; jy = jfy + c.hFy; jz = jfz + c.hFz; }
    rho_out = rho; jx_out = jx; jy_out = jy; jz_out = jz;

    const R ux = jx * c.invS, uy = jy * c.invS, uz = jz * c.invS;   // true velocity
    const R jxux = jx * ux, jyuy = jy * uy, jzuz = jz * uz;
    const R ju = jxux + jyuy + jzuz;                                 // S |u|^2

    // moment-space forcing MF = M Fbar (scaled)
    R A, P, Wf, Qxy, Qyz, Qxz;
    if (YF) {
        A = jy * c.Fy;                    // S u.F
        P = -A;                           // MF_3pxx / 2
        Wf = A;                           // MF_pww / 2
        Qxy = jx * c.Fy;
        Qyz = jz * c.Fy;
        Qxz = R(0);
    } else {
        A = jx * c.Fx + jy * c.Fy + jz * c.Fz;
        P = R(2) * (jx * c.Fx) - jy * c.Fy - jz * c.Fz;
        Wf = jy * c.Fy - jz * c.Fz;
        Qxy = jx * c.Fy + jy * c.Fx;
        Qyz = jy * c.Fz + jz * c.Fy;
        Qxz = jx * c.Fz + jz * c.Fx;
    }

    // raw moments of f (non-conserved)
    const R e   = R(-30) * f[0] + R(-11) * sa + R(8) * sd;
    const R eps = R(12) * f[0] + R(-4) * sa + sd;
    const R qx = R(-4) * d1 + Dx, qy = R(-4) * d3 + Dy, qz = R(-4) * d5 + Dz;
    const R t_yz = R(2) * syz;
    const R p3  = (R(2) * s1 - syz5) + (sxyz - t_yz);     // 3 p_xx
    const R pi3 = (R(2) * syz5 - R(4) * s1) + (sxyz - t_yz);  // 3 pi_xx
    const R s35 = s3 - s5, sxy_xz = sxy - sxz;
    const R pw  = s35 + sxy_xz;                            // p_ww
    const R piw = R(-2) * s35 + sxy_xz;                    // pi_ww
    const R pxy = s7 - s8, pyz = s15 - s16, pxz = s11 - s12;
    const R mx = (d7 - d8) - (d11 - d12);
    const R my = (d15 - d16) - (d7 + d8);
    const R mz = (d11 + d12) - (d15 + d16);

    // equilibria (scaled) of the moments that depend on j
    const R eqp = R(3) * jxux - ju;          // 3 p_xx
    const R eqw = jyuy - jzuz;               // p_ww

    // increments a_k = (MF_k - s_k (m_k + MF_k/2 - meq_k)) / d_k
    const R a_e   = A * R(38.0 / 2394.0) - c.ke * (e + R(19) * A + R(11) * rho - R(19) * ju);
    const R a_eps = A * R(-11.0 / 252.0) - c.keps * (eps - R(5.5) * A - c.oeps * rho - c.oepsj * ju);
    R a_qx, a_qz;
    if (YF) {
        a_qx = -c.kq * (qx + R(2.0 / 3.0) * jx);
        a_qz = -c.kq * (qz + R(2.0 / 3.0) * jz);
    } else {
        a_qx = c.fqx - c.kq * (qx + R(2.0 / 3.0) * jx - c.thFx);
        a_qz = c.fqz - c.kq * (qz + R(2.0 / 3.0) * jz - c.thFz);
    }
    const R a_qy = c.fqy - c.kq * (qy + R(2.0 / 3.0) * jy - c.thFy);
    const R a_p  = P * R(2.0 / 36.0) - c.kp * (p3 + P - eqp);
    const R a_pi = P * R(-1.0 / 72.0) - c.kpi * (pi3 - R(0.5) * P - c.oxx * eqp);
    const R a_w  = Wf * R(2.0 / 12.0) - c.kw * (pw + Wf - eqw);
    const R a_wi = Wf * R(-1.0 / 24.0) - c.kwi * (piw - R(0.5) * Wf - c.oxx * eqw);
    const R a_xy = Qxy * R(0.25) - c.kxy * (pxy + R(0.5) * Qxy - jx * uy);
    const R a_yz = Qyz * R(0.25) - c.kxy * (pyz + R(0.5) * Qyz - jy * uz);
    const R a_xz = YF ? -c.kxy * (pxz - jx * uz) : Qxz * R(0.25) - c.kxy * (pxz + R(0.5) * Qxz - jx * uz);
    const R a_mx = -c.km * mx, a_my = -c.km * my, a_mz = -c.km * mz;

    R ajx, ajy, ajz;
    if (FROZEN) {
        // back-transform conserves the frozen j + S F/2 instead of sum c f + S F
        ajx = (jx + c.hFx - jfx) * R(0.1);
        ajy = (jy + c.hFy - jfy) * R(0.1);
        ajz = (jz + c.hFz - jfz) * R(0.1);
    } else {
        ajx = c.ajx; ajy = c.ajy; ajz = c.ajz;
    }
    // with a streamwise-only force the x and z momentum increments vanish
    const R Ox = YF && !FROZEN ? R(-4) * a_qx : ajx - R(4) * a_qx;
    const R Oz = YF && !FROZEN ? R(-4) * a_qz : ajz - R(4) * a_qz;
    const R gx = YF && !FROZEN ? a_qx : ajx + a_qx;
    const R gz = YF && !FROZEN ? a_qz : ajz + a_qz;

    // back-transform f* = f + M^T a
    f[0] += R(-30) * a_e + R(12) * a_eps;

    const R ba = R(-11) * a_e - R(4) * a_eps;
    const R Ex = ba + R(2) * a_p - R(4) * a_pi;
    const R Eyz = ba - a_p + R(2) * a_pi;
    const R tw = a_w - R(2) * a_wi;
    const R Ey = Eyz + tw, Ez = Eyz - tw;
    const R Oy = ajy - R(4) * a_qy;
    f[1] += Ex + Ox;  f[2] += Ex - Ox;
    f[3] += Ey + Oy;  f[4] += Ey - Oy;
    f[5] += Ez + Oz;  f[6] += Ez - Oz;

    const R bd = R(8) * a_e + a_eps;
    const R ppi = a_p + a_pi, wwi = a_w + a_wi;
    const R Exy = bd + ppi + wwi;
    const R Exz = bd + ppi - wwi;
    const R Eyy = bd - R(2) * ppi;
    const R gy = ajy + a_qy;

    // odd parts of the diagonal pairs share g +- a_m combinations
    const R uxm = gx + a_mx, uxp = gx - a_mx;
    const R uyp = gy - a_my, uym = gy + a_my;
    const R uzm = gz + a_mz, uzp = gz - a_mz;
    {   // 7 (+1,+1,0) / 10 and 8 (-1,+1,0) / 9
        const R E7 = Exy + a_xy, O7 = uxm + uyp;
        const R E8 = Exy - a_xy, O8 = uyp - uxm;
        f[7] += E7 + O7;  f[10] += E7 - O7;
        f[8] += E8 + O8;  f[9] += E8 - O8;
    }
    {   // 11 (+1,0,+1) / 14 and 12 (-1,0,+1) / 13
        const R E11 = Exz + a_xz, O11 = uxp + uzm;
        const R E12 = Exz - a_xz, O12 = uzm - uxp;
        f[11] += E11 + O11; f[14] += E11 - O11;
        f[12] += E12 + O12; f[13] += E12 - O12;
    }
    {   // 15 (0,+1,+1) / 18 and 16 (0,-1,+1) / 17
        const R E15 = Eyy + a_yz, O15 = uym + uzp;
        const R E16 = Eyy - a_yz, O16 = uzp - uym;
        f[15] += E15 + O15; f[18] += E15 - O15;
        f[16] += E16 + O16; f[17] += E16 - O16;
    }
}

}  // namespace lbm
