// host_io.cpp -- result files in the WAMIT formats the reference writes
// (Hydrodynamic_Solver_IO.cpp:430-646): .1 added mass / damping, .2 Haskind
// excitation, .2fk Froude-Krylov, .2sc scattering, .4 RAO, .hst hydrostatic
// stiffness, .mmx mass matrix.  Host only.
#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/bemgpu.h"

namespace {

const double kGravity = 9.81;  // the reference's global Gravity (BEMUse_Math_Types.h)
const double kR2D = 180.0 / M_PI;

// Number field: default stream formatting (6 significant digits), a leading blank
// for non-negative values, right-padded with blanks to `pad` characters
// (PFS, BEMUse_IO.h:58-67).
std::string num(double a, int pad = 15) {
    std::ostringstream s;
    s << a;
    std::string o = s.str();
    if (a >= 0) o.insert(0, " ");
    if ((int)o.size() < pad) o.append(pad - o.size(), ' ');
    return o;
}

std::complex<double> cget(const double* v, int f, int i, int b, int nb) {
    const size_t o = 2 * ((size_t)f * 6 * nb + (size_t)i * nb + b);
    return {v[o], v[o + 1]};
}

}  // namespace

extern "C" bem_status bem_write_wamit(const char* prefix, const bem_wamit_info* info, int n_freq,
                                      const double* omega, const bem_result* r) {
    if (!prefix || !info || n_freq < 0 || (n_freq > 0 && (!omega || !r))) return BEM_ERR_ARG;
    const int nb = info->n_beta;
    if (nb < 0 || (nb > 0 && !info->betas)) return BEM_ERR_ARG;
    const std::string p(prefix);
    const double twopi = 2.0 * M_PI;
    // Frequency column: the reference prints its input Frequency = 2 pi Omega (Hydrodynamic_Solver.cpp:405).
    {
        std::ofstream f(p + ".hst", std::ios::trunc);
        if (!f) return BEM_ERR_ARG;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j)
                f << "     " << i + 1 << "     " << j + 1 << "   " << num(info->C[6 * i + j] / info->rho / kGravity)
                  << "\n";
    }
    {
        std::ofstream f(p + ".mmx", std::ios::trunc);
        if (!f) return BEM_ERR_ARG;
        f << "\n";
        f << "Gravity:     " << info->gravity << "     Length scale:        1.00000\n";
        f << "\n";
        f << "Volume     " << info->volume << "\n";
        f << "Center of Buoyancy (Xb,Yb,Zb):   " << num(info->cob[0]) << num(info->cob[1]) << num(info->cob[2]) << "\n";
        f << "Center of Gravity  (Xg,Yg,Zg):   " << num(info->cog[0]) << num(info->cog[1]) << num(info->cog[2]) << "\n";
        f << "\n";
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j)
                f << "     " << i + 1 << "     " << j + 1 << "   " << num(info->M[6 * i + j] / info->rho) << "\n";
    }
    std::ofstream f1(p + ".1", std::ios::trunc), f2(p + ".2", std::ios::trunc), ffk(p + ".2fk", std::ios::trunc),
        fsc(p + ".2sc", std::ios::trunc), f4(p + ".4", std::ios::trunc);
    if (!f1 || !f2 || !ffk || !fsc || !f4) return BEM_ERR_ARG;
    for (int k = 0; k < n_freq; ++k) {
        const double Om = omega[k], freq = twopi * Om;
        if (r->A && r->B)
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) {
                    const double a = r->A[36 * (size_t)k + 6 * i + j], b = r->B[36 * (size_t)k + 6 * i + j];
                    if (Om == 0.0)
                        f1 << num(0.0) << i + 1 << "     " << j + 1 << "     " << num(a) << "\n";
                    else
                        f1 << num(freq) << i + 1 << "     " << j + 1 << "     " << num(a) << num(b) << "\n";
                }
        if (Om == 0.0) continue;  // no incident wave
        struct Out { std::ofstream* s; const double* v; double scale; bool conj; };
        const Out outs[4] = {{&f2, r->F, kGravity, false}, {&ffk, r->FK, kGravity, false},
                             {&fsc, r->SC, kGravity, true}, {&f4, r->RAO, 1.0, false}};
        for (const Out& o : outs) {
            if (!o.v) continue;
            for (int b = 0; b < nb; ++b)
                for (int i = 0; i < 6; ++i) {
                    std::complex<double> z = cget(o.v, k, i, b, nb);
                    if (o.conj) z = std::conj(z);  // the .2sc file carries -arg and -Im (Hydrodynamic_Solver_IO.cpp:567-569)
                    *o.s << num(freq) << num(info->betas[b] * kR2D) << i + 1 << "  " << num(std::abs(z) / o.scale)
                         << num(std::arg(z)) << num(z.real() / o.scale) << num(z.imag() / o.scale) << "\n";
                }
        }
    }
    return BEM_OK;
}
