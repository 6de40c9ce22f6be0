// Host-side set-up of the C ABI: parameter derivation, domain walls and the
// inlet velocity profile.  Compiled by the host compiler with
// -ffp-contract=off so the T_P arithmetic is the reference's on every host.
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/mflbm.h"

namespace {

inline float pw(float a, float b) { return powf(a, b); }
inline double pw(double a, double b) { return pow(a, b); }

bool open_z(const mflbm_control* c) {
    return c->kper == 0 && c->domain_wall_status_z_min == 0 && c->domain_wall_status_z_max == 0;
}

// read_parameter_multi checks and derivations (src/IO_multiphase.cpp:198-242)
// and initialization_basic_multi (src/Init_multiphase.cpp:168-205, 258-269), in T.
template <class T>
void derive(const mflbm_control* ctl, int precision, int fp_mode, mflbm_params* o, mflbm_derived* d) {
    const T Pi = T(3.14159265358979323846);
    std::memset(o, 0, sizeof(*o));
    o->nx = ctl->nxGlobal;
    o->ny = ctl->nyGlobal;
    o->nz = ctl->nzGlobal;
    o->precision = precision;
    o->fp_mode = fp_mode;
    o->jper = ctl->jper;
    o->kper = ctl->kper;
    o->domain_wall_status_z_min = ctl->domain_wall_status_z_min;
    o->domain_wall_status_z_max = ctl->domain_wall_status_z_max;
    o->inlet_BC = ctl->inlet_BC;
    o->outlet_BC = ctl->outlet_BC;
    o->porous_plate_cmd = ctl->porous_plate_cmd;
    o->Z_porous_plate = ctl->Z_porous_plate;
    T theta = T(180) - T(ctl->theta);           // measured through the defending phase
    theta = theta * Pi / T(180);
    o->cos_theta = (double)(T)std::cos(theta);
    const T nu1 = T(ctl->fluid1_viscosity), nu2 = T(ctl->fluid2_viscosity), gamma = T(ctl->surface_tension);
    o->lbm_gamma = (double)gamma;
    o->lbm_beta = (double)T(ctl->RK_beta);
    o->la_nui1 = (double)(T(1) / nu1);
    o->la_nui2 = (double)(T(1) / nu2);
    const T sa = T(ctl->saturation_injection);
    o->sa_inject = (double)sa;
    o->phi_inlet = (double)(T(2) * sa - T(1));
    o->relaxation = 1.0;
    const T force_z0 = T(ctl->body_force_0);
    T force_z = force_z0, rho_out = T(1), rho_in = T(0), uin_avg = T(0), uin_avg_0 = T(0), flowrate = T(0);
    const T la_y = T(ctl->nyGlobal - 1) - T(0.5) - T(0.5);
    const T la_x = T(ctl->nxGlobal - 1) - T(0.5) - T(0.5);
    const T A_xy = la_x * la_y;
    if (open_z(ctl)) {
        if (ctl->inlet_BC == 1) {
            force_z = T(0);
            uin_avg_0 = T(ctl->capillary_number) * gamma / nu1;
            uin_avg = uin_avg_0;
            flowrate = uin_avg_0 * A_xy;
        } else if (ctl->inlet_BC == 2) {
            force_z = T(0);
            const T p_gradient = -force_z0 / T(3);
            if (ctl->rho_out_BC) rho_out = T(1) - p_gradient * T(ctl->nzGlobal);
            else rho_in = rho_out - p_gradient * T(ctl->nzGlobal);
        }
    }
    o->force_z = (double)force_z;
    o->uin_avg = (double)uin_avg;
    o->rho_in = (double)rho_in;
    o->rho_out = (double)rho_out;
    if (d) {
        d->A_xy = (double)A_xy;
        d->uin_avg_0 = (double)uin_avg_0;
        d->flowrate = (double)flowrate;
        d->interface_z0 = (double)T(ctl->initial_interface_position);
    }
}

// Uniform interior profile, then the analytic rectangular-duct profile with
// 1000 series terms (src/Init_multiphase.cpp:270-284, src/Misc.cpp:387-419).
template <class T>
void inlet_profile(const mflbm_control* ctl, T* W) {
    const long long nx = ctl->nxGlobal, ny = ctl->nyGlobal;
    const long long NX1 = nx + 2;
    for (long long n = 0; n < (nx + 2) * (ny + 2); ++n) W[n] = T(0);
    if (!(open_z(ctl) && ctl->inlet_BC == 1)) return;
    mflbm_params p;
    mflbm_derived d;
    derive<T>(ctl, sizeof(T) == 4 ? MFLBM_FP32 : MFLBM_FP64, 0, &p, &d);
    const T Pi = T(3.14159265358979323846);
    for (long long j = 1; j <= ny; ++j)
        for (long long i = 1; i <= nx; ++i) W[i + NX1 * j] = (i > 1 && i < nx && j > 1 && j < ny) ? T(p.uin_avg) : T(0);
    const T vel = T(d.uin_avg_0);
    const T la_y = T(ny - 1) - T(0.5) - T(0.5), la_x = T(nx - 1) - T(0.5) - T(0.5);
    const T a = T(0.5) * la_x, b = T(0.5) * la_y;
    T s1 = T(0);
    for (long long n = 1; n <= 1000; n += 2) s1 += (std::tanh(T(0.5) * T(n) * Pi * b / a)) / pw(T(n), T(5));
    T s2 = T(1) - T(192) / pw(Pi, T(5)) * (a / b) * s1;
    s2 = T(-3) * vel / (s2 * pw(a, T(2)));
    for (long long j = 2; j < ny; ++j)
        for (long long i = 2; i < nx; ++i) {
            const T xx = T(i) - T(1.5) - a, yy = T(j) - T(1.5) - b;
            T s3 = T(0);
            for (long long n = 1; n <= 1000; n += 2)
                s3 += pw(T(-1), T(0.5) * T((n - 1))) * std::cos(T(0.5) * T(n) * Pi * xx / a) / pw(T(n), T(3)) *
                      (T(1) - (std::exp(T(0.5) * T(n) * Pi * (yy - b) / a) + std::exp(T(0.5) * T(n) * Pi * (-yy - b) / a)) /
                                  (T(1) + std::exp(T(0.5) * T(n) * Pi * (-b - b) / a)));
            W[i + NX1 * j] = s3 * (T(-16) * s2 * pw(a, T(2)) * pw(Pi, T(-3)));
        }
}

}  // namespace

namespace mflbm {
int fail(int code, const std::string& msg);
}

extern "C" int mflbm_params_from_control(const mflbm_control* ctl, int precision, int fp_mode, mflbm_params* out,
                                         mflbm_derived* derived) {
    if (!ctl || !out) return mflbm::fail(MFLBM_E_ARG, "mflbm_params_from_control: null pointer");
    if (precision != MFLBM_FP32 && precision != MFLBM_FP64)
        return mflbm::fail(MFLBM_E_ARG, "mflbm_params_from_control: precision must be MFLBM_FP32 or MFLBM_FP64");
    if (ctl->theta > 90.0)
        return mflbm::fail(MFLBM_E_ARG, "contact angle is larger than 90 degrees");
    if (ctl->iper == 1 || ctl->domain_wall_status_x_max == 0 || ctl->domain_wall_status_x_min == 0)
        return mflbm::fail(MFLBM_E_ARG, "x must be walled and non-periodic");
    if (ctl->jper == 0 && (ctl->domain_wall_status_y_max == 0 || ctl->domain_wall_status_y_min == 0))
        return mflbm::fail(MFLBM_E_ARG, "y walls missing while y is not periodic");
    if (ctl->jper == 1 && (ctl->domain_wall_status_y_max == 1 || ctl->domain_wall_status_y_min == 1))
        return mflbm::fail(MFLBM_E_ARG, "y walls present while y is periodic");
    if (ctl->kper == 1 && (ctl->domain_wall_status_z_max == 1 || ctl->domain_wall_status_z_min == 1))
        return mflbm::fail(MFLBM_E_ARG, "z walls present while z is periodic");
    if (ctl->outlet_BC == 1 && ctl->inlet_BC == 2)
        return mflbm::fail(MFLBM_E_ARG, "pressure inlet + convective outlet is not supported");
    if (precision == MFLBM_FP32) derive<float>(ctl, precision, fp_mode, out, derived);
    else derive<double>(ctl, precision, fp_mode, out, derived);
    return MFLBM_OK;
}

extern "C" int mflbm_set_walls(const mflbm_control* ctl, const uint8_t* geo, int32_t* wg) {
    if (!ctl || !wg) return mflbm::fail(MFLBM_E_ARG, "mflbm_set_walls: null pointer");
    const long long nx = ctl->nxGlobal, ny = ctl->nyGlobal, nz = ctl->nzGlobal;
    if (geo && nx != ny) return mflbm::fail(MFLBM_E_ARG, "geometry files need nx == ny");
    auto s0 = [&](long long x, long long y, long long z) { return (x - 1) + nx * ((y - 1) + ny * (z - 1)); };
    for (long long k = 1; k <= nz; ++k)
        for (long long j = 1; j <= ny; ++j)
            for (long long i = 1; i <= nx; ++i)
                wg[s0(i, j, k)] = geo ? (int32_t)geo[(i - 1) + ny * ((j - 1) + nx * (k - 1))] : 0;
    for (long long k = 1; k <= nz; ++k)
        for (long long j = 1; j <= ny; ++j)
            for (long long i = 1; i <= nx; ++i) {
                if (ctl->domain_wall_status_z_min == 1) wg[s0(i, j, 1)] = 1;
                if (ctl->domain_wall_status_z_max == 1) wg[s0(i, j, nz)] = 1;
                if (ctl->domain_wall_status_x_min == 1) wg[s0(1, j, k)] = 1;
                if (ctl->domain_wall_status_x_max == 1) wg[s0(nx, j, k)] = 1;
                if (ctl->domain_wall_status_y_min == 1) wg[s0(i, 1, k)] = 1;
                if (ctl->domain_wall_status_y_max == 1) wg[s0(i, ny, k)] = 1;
            }
    return MFLBM_OK;
}

extern "C" int mflbm_inlet_profile(const mflbm_control* ctl, int precision, void* W_in) {
    if (!ctl || !W_in) return mflbm::fail(MFLBM_E_ARG, "mflbm_inlet_profile: null pointer");
    if (precision == MFLBM_FP32) inlet_profile<float>(ctl, (float*)W_in);
    else if (precision == MFLBM_FP64) inlet_profile<double>(ctl, (double*)W_in);
    else return mflbm::fail(MFLBM_E_ARG, "mflbm_inlet_profile: bad precision");
    return MFLBM_OK;
}
