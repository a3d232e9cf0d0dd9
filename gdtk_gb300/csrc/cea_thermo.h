// cea_thermo.h -- NASA-9 (CEA) species thermo shared by the kernels and by the host-side table
// preparation (the extrapolation constants Cp/h/s at the curve ends).  Restates
// gas/thermo/cea_thermo_curves.d:55-182 in its evaluation order.
#pragma once
#include <cmath>
#include "chem_types.h"

namespace gdtk {

// ---------------------------------------------------------------- thermo (CEA / NASA-9)
// cea_thermo_curves.d:150-182.  Returns false when no segment applies (T is NaN).
GDTK_HD bool cea_coeffs(const MechView& m, int isp, double T, double a[9]) {
    const double* s = m.sp(isp);
    const int nseg = m.nseg(isp);
    const double* br = s + SP_BREAKS;
    const double* bl = s + SP_BLENDS;
    const double* co = s + SP_COEFFS;
    if (nseg == 1) {
        if (T != T) return false;
#pragma unroll
        for (int j = 0; j < 9; ++j) a[j] = co[j];
        return true;
    }
    const int nb = nseg + 1, nbl = nseg - 1;
    if (T < (br[1] - 0.5 * bl[0])) {
#pragma unroll
        for (int j = 0; j < 9; ++j) a[j] = co[j];
        return true;
    }
    if (T > (br[nb - 2] + 0.5 * bl[nbl - 1])) {
#pragma unroll
        for (int j = 0; j < 9; ++j) a[j] = co[(nseg - 1) * 9 + j];
        return true;
    }
    for (int i = 1; i < nb - 1; ++i) {
        double T_blend_low = br[i] - 0.5 * bl[i - 1];
        double T_blend_high = br[i] + 0.5 * bl[i - 1];
        if (T >= T_blend_low && T <= T_blend_high) {
            double wB = (1. / bl[i - 1]) * (T - T_blend_low);
            double wA = 1.0 - wB;
#pragma unroll
            for (int j = 0; j < 9; ++j) a[j] = wA * co[(i - 1) * 9 + j] + wB * co[i * 9 + j];
            return true;
        }
        if (T > T_blend_high && i < nbl && T < (br[i + 1] - 0.5 * bl[i])) {
#pragma unroll
            for (int j = 0; j < 9; ++j) a[j] = co[i * 9 + j];
            return true;
        }
    }
    return false;
}

GDTK_HD double cea_Cp(const MechView& m, int isp, double T, int& err) {
    const double* s = m.sp(isp);
    if (T < s[SP_TLOW]) return s[SP_CPLOW];
    if (T > s[SP_THIGH]) return s[SP_CPHIGH];
    double a[9];
    if (!cea_coeffs(m, isp, T, a)) { err = CELL_CEA_RANGE; return 0.0; }
    double Cp_on_R = a[0] / (T * T) + a[1] / T + a[2] + a[3] * T;
    Cp_on_R += a[4] * T * T + a[5] * T * T * T + a[6] * T * T * T * T;
    return s[SP_R] * Cp_on_R;
}

GDTK_HD double cea_h(const MechView& m, int isp, double T, double logT, int& err) {
    const double* s = m.sp(isp);
    if (T < s[SP_TLOW]) return s[SP_HLOW] - s[SP_CPLOW] * (s[SP_TLOW] - T);
    if (T > s[SP_THIGH]) return s[SP_HHIGH] + s[SP_CPHIGH] * (T - s[SP_THIGH]);
    double a[9];
    if (!cea_coeffs(m, isp, T, a)) { err = CELL_CEA_RANGE; return 0.0; }
    double h_on_RT = -a[0] / T + a[1] * logT + a[2] * T + a[3] * T * T / 2.0;
    h_on_RT += a[4] * T * T * T / 3.0 + a[5] * T * T * T * T / 4.0 + a[6] * T * T * T * T * T / 5.0 + a[7];
    return s[SP_R] * h_on_RT;
}

GDTK_HD double cea_s(const MechView& m, int isp, double T, double logT, int& err) {
    const double* s = m.sp(isp);
    if (T < s[SP_TLOW]) return s[SP_SLOW] - s[SP_CPLOW] * log(s[SP_TLOW] / T);
    if (T > s[SP_THIGH]) return s[SP_SHIGH] + s[SP_CPHIGH] * log(T / s[SP_THIGH]);
    double a[9];
    if (!cea_coeffs(m, isp, T, a)) { err = CELL_CEA_RANGE; return 0.0; }
    double s_on_R = -a[0] / (2.0 * T * T) - a[1] / T + a[2] * logT + a[3] * T;
    s_on_R += a[4] * T * T / 2.0 + a[5] * T * T * T / 3.0 + a[6] * T * T * T * T / 4.0 + a[8];
    return s[SP_R] * s_on_R;
}

}  // namespace gdtk
