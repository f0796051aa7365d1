/*
 * settings.cpp -- defaults of SIM / FLUID / AERO / INTEG_SETT (src/Var.h:63-394) and the
 * derivations of Set_Values (src/IO.cpp:26-128), host code behind the C ABI.
 */
#include <cmath>
#include <cstring>

#include "../../include/fjsph_gb300.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

/* Kernel.h:37-45 / :11-21 */
double kernel_value(double dist, double H, double Wc, bool cubic) {
    if (cubic) {
        double q = dist / H;
        if (q < 1.0) return Wc * (1.0 - 1.5 * q * q * (1 - 0.5 * q));
        if (q < 2.0) return Wc * 0.25 * std::pow(2.0 - q, 3.0);
        return 0.0;
    }
    return std::pow(1 - 0.5 * dist / H, 4) * (2 * dist / H + 1) * Wc;
}

/* get_n_full (src/Geometry.cpp:282-308): lattice points within the search radius of the origin,
 * the lattice walked from -2(H+dx) to 2(H+dx) by accumulating dx as the reference does. */
double n_full_count(double dx, double H, int D) {
    const double sr = 4.0 * H * H;
    const double lim = 2.0 * (H + dx);
    long count = 0;
    for (double x = -lim; x <= lim; x += dx)
        for (double y = -lim; y <= lim; y += dx) {
            if (D == 3) {
                for (double z = -lim; z <= lim; z += dx) {
                    double r = x * x;
                    r = std::fma(y, y, r);
                    r = std::fma(z, z, r);
                    if (r < sr) ++count;
                }
            } else {
                double r = x * x;
                r = std::fma(y, y, r);
                if (r < sr) ++count;
            }
        }
    return double(count);
}

double eos_density(const fjsph_settings *s, double press) {
    if (s->pressure_rel == FJSPH_ISO_EOS) return (press - s->press_back) / (s->speed_sound * s->speed_sound) + s->rho_rest;
    return s->rho_rest * std::pow(((press - s->press_back) / s->B) + 1.0, 1.0 / s->gam);
}

} // namespace

extern "C" int fjsph_settings_defaults(fjsph_settings *s, int32_t dim) {
    if (!s || (dim != 2 && dim != 3)) return FJSPH_E_ARG;
    std::memset(s, 0, sizeof(*s));
    s->dim = dim;
    s->variant = 0;
    s->st_model = FJSPH_ST_PAIRWISE;
    s->precision = FJSPH_PREC_FP64;
    s->aero_closure = FJSPH_CLOSURE_PLAIN;
    s->solver_type = FJSPH_NEWMARK_BETA;
    /* FLUID (Var.h:160-200) */
    s->pressure_rel = FJSPH_COLE_EOS;
    s->H = -1.0;
    s->H_sq = -1.0;
    s->sr = -1.0;
    s->H_fac = 2.0;
    s->W_dx = -1.0;
    s->rho_rest = 1000.0;
    s->rho_pipe = 1000.0;
    s->press_pipe = 0.0;
    s->press_back = 0.0;
    s->rho_max = 1500.0;
    s->rho_min = 500.0;
    s->rho_var = 50.0;
    s->rho_max_iter = 1.0;
    s->sim_mass = -1.0;
    s->bnd_mass = -1.0;
    s->W_correc = -1.0;
    s->visc_alpha = 0.1;
    s->speed_sound = 300.0;
    s->mu = 8.94e-4;
    s->nu = s->mu / s->rho_rest;
    s->sig = 0.0708;
    s->gam = 7.0;
    s->B = -1.0;
    s->contangb = 150.0;
    s->dsph_delta = 0.1;
    s->dsph_cont = -1.0;
    /* SIM (Var.h:337-394) */
    s->particle_step = -1.0;
    s->dx = -1.0;
    s->scale = 1.0;
    s->grav[0] = 0.0;
    s->grav[1] = dim == 3 ? 0.0 : -9.81;
    s->grav[2] = dim == 3 ? -9.81 : 0.0;
    s->asource = 0;
    s->init_hydro_pressure = 0;
    s->hydro_height = -1.0;
    s->max_points = 9999999;
    /* AERO (Var.h:240-310) */
    s->acase = FJSPH_NOAERO;
    s->use_lam = 1;
    s->use_TAB_def = 0;
    s->use_dx = 0;
    s->L = s->td = s->omega = s->tmax = s->ycoef = -1.0;
    s->Cf = 1.0 / 3.0;
    s->Ck = 8.0;
    s->Cd = 5.0;
    s->Cb = 0.5;
    s->Cdef = -1.0;
    s->A_sphere = s->A_plate = -1.0;
    s->v_ref = 0.0;
    s->p_ref = 101353.0;
    s->rho_g = 1.29251;
    s->mu_g = 1.716e-5;
    s->mass_g = -1.0;
    s->temp_g = 298.0;
    s->R_g = 287.0;
    s->gamma_g = 1.403;
    s->sos = std::sqrt(s->temp_g * s->R_g * s->gamma_g);
    s->i_sos_sq = 1.0 / (s->sos * s->sos);
    s->M_ref = -1.0;
    s->lam_cutoff = 0.75;
    s->interp_fac = 2.0;
    s->i_interp_fac = 0.5;
    s->n_full = dim == 2 ? 30 : 200;
    s->i_n_full = 1.0 / s->n_full;
    s->i_n_count = 1.0 / (s->i_interp_fac * s->n_full);
    /* INTEG_SETT (Var.h:63-92) */
    s->max_subits = 20;
    s->n_stable = 0;
    s->n_stable_limit = 10;
    s->n_unstable = 0;
    s->n_unstable_limit = 3;
    s->subits_factor = 0.333;
    s->cfl = 1.0;
    s->cfl_step = 0.05;
    s->cfl_max = 2.0;
    s->cfl_min = 0.1;
    s->current_time = 0.0;
    s->last_frame_time = 0.0;
    s->frame_time_interval = 1e30; /* must come from the para file upstream */
    s->min_residual = -7.0;
    s->delta_t = 2e-10;
    s->delta_t_max = 1.0;
    s->delta_t_min = 0.0;
    s->nb_beta = 0.25;
    s->nb_gamma = 0.5;
    s->max_shift_vel = 9999999;
    s->reorder_interval = 8;
    s->learned_judge_interval = 50;
    return FJSPH_OK;
}

/* Set_Values (src/IO.cpp:26-128) and AERO::GetYcoef (src/Var.h:244-266). */
extern "C" int fjsph_settings_derive(fjsph_settings *s) {
    if (!s || (s->dim != 2 && s->dim != 3) || !(s->particle_step > 0)) return FJSPH_E_ARG;
    const int D = s->dim;
    const bool cubic = (s->variant & FJSPH_VAR_CUBIC) != 0;
    s->B = s->rho_rest * std::pow(s->speed_sound, 2) / s->gam;
    s->rho_pipe = eos_density(s, s->press_pipe);
    if (s->rho_max == 1500 && s->rho_min == 500) {
        s->rho_max = s->rho_rest * (1.0 + s->rho_var * 0.01);
        s->rho_min = s->rho_rest * (1.0 - s->rho_var * 0.01);
    }
    s->dx = s->particle_step * std::pow(s->rho_pipe / s->rho_rest, 1.0 / D);
    s->nb_beta = 0.25;
    s->nb_gamma = 0.5;
    s->sim_mass = s->rho_rest * std::pow(s->particle_step, D);
    s->bnd_mass = s->sim_mass;
    s->mass_g = s->rho_g * std::pow(s->particle_step, D);
    s->sos = std::sqrt(s->temp_g * s->R_g * s->gamma_g);
    s->i_sos_sq = 1.0 / (s->sos * s->sos);
    if (s->M_ref != -1)
        s->v_ref = s->sos * s->M_ref;
    else
        s->M_ref = s->v_ref / s->sos;
    s->delta_t = s->delta_t_min > 0 ? s->delta_t_min : 2e-10;
    s->H = s->H_fac * s->particle_step;
    s->H_sq = s->H * s->H;
    s->sr = 4 * s->H_sq;
    s->dsph_cont = 2.0 * s->dsph_delta * s->H * s->speed_sound;
    s->nu = s->mu / s->rho_rest;
    if (D == 2)
        s->W_correc = cubic ? 10.0 / (7.0 * kPi * s->H * s->H) : 7.0 / (4.0 * kPi * s->H * s->H);
    else
        s->W_correc = cubic ? (1.0 / (kPi * s->H * s->H * s->H)) : (21 / (16 * kPi * s->H * s->H * s->H));
    s->W_dx = kernel_value(s->particle_step, s->H, s->W_correc, cubic);
    /* GetYcoef */
    const double diam = s->particle_step;
    if (D == 3) {
        s->L = diam * std::cbrt(3.0 / (4.0 * kPi));
        s->A_sphere = kPi * s->L * s->L;
        s->A_plate = diam * diam;
    } else {
        s->L = diam / std::sqrt(kPi);
        s->A_sphere = 2 * s->L;
        s->A_plate = diam;
    }
    s->td = (2.0 * s->rho_rest * std::pow(s->L, D - 1)) / (s->Cd * s->mu);
    s->omega = std::sqrt((s->Ck * s->sig) / (s->rho_rest * std::pow(s->L, D)) - 1.0 / std::pow(s->td, 2.0));
    s->tmax = -2.0 * (std::atan(std::sqrt(std::pow(s->td * s->omega, 2.0) + 1) + s->td * s->omega) - kPi) / s->omega;
    s->Cdef = 1.0 - std::exp(-s->tmax / s->td) *
                        (std::cos(s->omega * s->tmax) + 1 / (s->omega * s->td) * std::sin(s->omega * s->tmax));
    s->ycoef = 0.5 * s->Cdef * (s->Cf / (s->Ck * s->Cb)) * (s->rho_g * s->L) / s->sig;
    s->n_full = n_full_count(s->particle_step, s->H, D);
    s->i_n_full = 1.0 / s->n_full;
    s->interp_fac = 1.0 / s->i_interp_fac;
    s->A_plate = D == 3 ? s->particle_step * s->particle_step : s->particle_step;
    return FJSPH_OK;
}

extern "C" int fjsph_abi_sizes(int64_t *sizes4) {
    if (!sizes4) return FJSPH_E_ARG;
    sizes4[0] = (int64_t)sizeof(fjsph_settings);
    sizes4[1] = (int64_t)sizeof(fjsph_block);
    sizes4[2] = (int64_t)sizeof(fjsph_inlet);
    sizes4[3] = (int64_t)sizeof(fjsph_state_view);
    return FJSPH_OK;
}
