// host_io.cpp -- result files in the WAMIT formats the reference writes
// (Hydrodynamic_Solver_IO.cpp:430-646): .1 added mass / damping, .2 Haskind
// excitation, .2fk Froude-Krylov, .2sc scattering, .4 RAO, .hst hydrostatic
// stiffness, .mmx mass matrix, the Kochin-function files and the free-surface
// elevation (.6r, _WaveElPos.bem); and the mesh importers.  Host only.
#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <algorithm>
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

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
    const int nk = info->n_kochin, nw = info->n_wave;
    if (nk < 0 || nw < 0 || (nw > 0 && !info->wave_points)) return BEM_ERR_ARG;
    std::ofstream f1(p + ".1", std::ios::trunc), f2(p + ".2", std::ios::trunc), ffk(p + ".2fk", std::ios::trunc),
        fsc(p + ".2sc", std::ios::trunc), f4(p + ".4", std::ios::trunc), f6(p + ".6", std::ios::trunc),
        fkr(p + "_KochinRad.bem", std::ios::trunc), fkd(p + "_KochinDiff.bem", std::ios::trunc);
    if (!f1 || !f2 || !ffk || !fsc || !f4 || !f6 || !fkr || !fkd) return BEM_ERR_ARG;
    std::ofstream f6r;
    if (nw > 0) {
        std::ofstream fp(p + "_WaveElPos.bem", std::ios::trunc);
        f6r.open(p + ".6r", std::ios::trunc);
        if (!fp || !f6r) return BEM_ERR_ARG;
        for (int i = 0; i < nw; ++i)
            fp << i << "     " << num(info->wave_points[3 * i]) << num(info->wave_points[3 * i + 1]) << "\n";
    }
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
        // Kochin functions (Hydrodynamic_Solver_IO.cpp:589-623), theta in degrees
        auto kget = [&](const double* v, int n, int i, int j) {
            const size_t o = 2 * (((size_t)k * nk + i) * n + j);
            return std::complex<double>(v[o], v[o + 1]);
        };
        auto kline = [&](std::ostream& s, std::complex<double> z) {
            s << num(std::abs(z)) << num(std::arg(z)) << num(z.real()) << num(z.imag()) << "\n";
        };
        if (r->kochin_rad)
            for (int i = 0; i < nk; ++i) {
                const double th = (0.5 + i) * twopi / nk;
                for (int d = 0; d < 6; ++d) {
                    fkr << num(freq) << d + 1 << "  " << num(th * kR2D);
                    kline(fkr, kget(r->kochin_rad, 6, i, d));
                }
            }
        if (r->kochin_diff)
            for (int d = 0; d < nb; ++d)
                for (int i = 0; i < nk; ++i) {
                    const double th = (0.5 + i) * twopi / nk;
                    fkd << num(freq) << num(info->betas[d] * kR2D) << "  " << num(th * kR2D);
                    kline(fkd, kget(r->kochin_diff, nb, i, d));
                }
        // radiation wave elevation at the wave points (:625-645): |eta| and phase per dof
        if (nw > 0 && r->fs_rad)
            for (int i = 0; i < nw; ++i) {
                f6r << num(freq) << i << "     ";
                for (int d = 0; d < 6; ++d) {
                    const size_t o = 2 * (((size_t)k * nw + i) * 6 + d);
                    const std::complex<double> z(r->fs_rad[o], r->fs_rad[o + 1]);
                    f6r << num(std::abs(z)) << num(std::arg(z));
                }
                f6r << "\n";
            }
    }
    return BEM_OK;
}

namespace {

// Text field padded with blanks to `pad` characters (PST, BEMUse_IO.h:69-74).
std::string txt(const std::string& t, int pad = 15) {
    std::string o = t;
    if ((int)o.size() < pad) o.append(pad - o.size(), ' ');
    return o;
}

}  // namespace

extern "C" bem_status bem_write_bem(const char* prefix, const bem_summary_info* info, int n_freq,
                                    const double* omega, const bem_result* r) {
    if (!prefix || !info || !info->w || n_freq < 0 || (n_freq > 0 && (!omega || !r))) return BEM_ERR_ARG;
    const bem_wamit_info& w = *info->w;
    const int nb = w.n_beta;
    if (nb < 0 || (nb > 0 && !w.betas)) return BEM_ERR_ARG;
    std::ofstream f(std::string(prefix) + ".bem", std::ios::trunc);
    if (!f) return BEM_ERR_ARG;
    f << "---------------------------------------------------------------\n";
    f << "------------------------ BEMUse Output ------------------------\n";
    f << "---------------------------------------------------------------\n\n";
    f << "------------ Environmental Parameters ------------\n";
    f << "Gravity:                 " << kGravity << " m s^{-2}.\n";
    f << "Density of Water:        " << 1025 << " kg m^{-3}.\n";
    f << "Atmospheric Pressure:    " << 101325.0 << " Pa.\n";
    f << "Water Depth:             Infinite.\n\n";
    f << "------------ Wave Parameters ------------\n";
    f << "Incoming wave angles: (deg)        ";
    for (int b = 0; b < nb; ++b) f << num(w.betas[b] * kR2D);
    f << "\n\n------------ Grid Summary ------------\n";
    f << (info->file_info ? info->file_info : "") << "\n";
    f << "Input Mesh has:          " << info->n_nodes << " nodes.\n";
    f << "Input Mesh has:          " << info->n_elems << " panels.\n";
    f << "Input Mesh has:          " << info->n_aux_elems << " auxiliary panels.\n\n";
    f << "------------ Geometry Summary ------------\n";
    f << "Nb: This is calculated by BEMUse with the approximation of flat surface panels.\n";
    f << "With increasing mesh refinement the values are expected to approach those of the continuous geometry.\n";
    f << "Volume:                  " << w.volume << " m^3.\n";
    f << "Surface area:            " << info->surface_area << " m^2.\n";
    f << "Mass:                    " << info->mass << " kg. (Assuming not pre-specified),\n";
    f << "Centre of Mass:          [" << w.cog[0] << ", " << w.cog[1] << ", " << w.cog[2] << "] m.\n";
    f << "Centre of Buoyancy:      [" << w.cob[0] << ", " << w.cob[1] << ", " << w.cob[2] << "] m.\n\n";
    f << "------------ Inertial Summary ------------\n\n";
    auto mat = [&](const char* title, const double* m) {
        f << title << " \n";
        for (int i = 0; i < 6; ++i) {
            f << "|";
            for (int j = 0; j < 6; ++j) f << num(m[6 * i + j]);
            f << " |\n";
        }
        f << "\n";
    };
    mat("Mass Matrix:", w.M);
    mat("Hydrostatic stiffness Matrix:", w.C);
    f << "------------ Output of Hydrodynamic Analysis: ------------\n\n\n";
    static const char* rows_ab[6] = {"Surge", "Sway", "Heave", "Roll", "Pitch", "Yaw"};
    static const char* rows_f[6] = {"Surge: ", "Sway: ", "Heave: ", "Pitch: ", "Roll: ", "Yaw: "};
    for (int k = 0; k < n_freq; ++k) {
        const double Om = omega[k], freq = 2.0 * M_PI * Om;
        f << "----------\n";
        f << "Frequency:       " << Om << " s^{-1}.\n";
        f << "Period:          " << 1.0 / freq << " s.\n";
        f << "Wavenumber:      " << Om * Om / kGravity << " m^{-1}.\n\n";
        f << txt("Motion") << txt(" A_x") << txt(" B_x") << txt(" A_y") << txt(" B_y") << txt(" A_z") << txt(" B_z")
          << txt(" A_pitch") << txt(" B_pitch") << txt(" A_roll") << txt(" B_roll") << txt(" A_yaw") << txt(" B_yaw")
          << "\n";
        for (int i = 0; i < 6; ++i) {
            f << txt(rows_ab[i]);
            for (int j = 0; j < 6; ++j) {
                const size_t o = 36 * (size_t)k + 6 * i + j;
                f << num(r->A ? r->A[o] : 0.0) << num(r->B ? r->B[o] : 0.0);
            }
            f << "\n";
        }
        f << "\n\n";
        std::string heading = txt("Wave Heading: (deg) ", 30);
        for (int b = 0; b < nb; ++b) heading += num(w.betas[b] * kR2D, 30);
        auto table = [&](const char* title, const double* v, const char* lab) {
            f << title << "\n" << heading << "\n" << txt("Motion: ", 30);
            for (int b = 0; b < nb; ++b) f << txt(std::string(" Mag(") + lab + ")") << txt(std::string(" Arg(") + lab + ")");
            f << "\n";
            for (int i = 0; i < 6; ++i) {
                f << txt(rows_f[i], 30);
                for (int b = 0; b < nb; ++b) {
                    const std::complex<double> z = v ? cget(v, k, i, b, nb) : std::complex<double>(0, 0);
                    f << num(std::abs(z) / kGravity) << num(std::arg(z));
                }
                f << "\n";
            }
            f << "\n\n";
        };
        table("Froude-Krylov Forces:", r->FK, "Fh");
        table("Excitation Forces:", r->F, "Xh");
        f << "----------\n\n";
    }
    return BEM_OK;
}

namespace {

// Blank-separated fields as the reference's Split(line, ' ') returns them
// (BEMUse_IO.h:11-26): runs of blanks separate fields and the text after the
// last blank is always a field, so a trailing blank adds an empty field and
// such a line never has exactly three.
std::vector<std::string> split_blank(const std::string& t) {
    std::vector<std::string> out;
    size_t start = 0, end;
    while ((end = t.find(' ', start)) != std::string::npos) {
        if (end != start) out.push_back(t.substr(start, end - start));
        start = end + 1;
    }
    out.push_back(t.substr(start));
    return out;
}

// std::stod / std::stoi semantics: leading white space skipped, trailing
// characters (a '\r' from a DOS line end, say) ignored, no digits is an error.
bool parse_double(const std::string& f, double& v) {
    char* e = nullptr;
    v = std::strtod(f.c_str(), &e);
    return e != f.c_str();
}

bool parse_int(const std::string& f, long& v) {
    char* e = nullptr;
    v = std::strtol(f.c_str(), &e, 10);
    return e != f.c_str();
}

bool parse_xyz(const std::vector<std::string>& fl, size_t at, double* v) {
    if (fl.size() < at + 3) return false;
    for (int c = 0; c < 3; ++c)
        if (!parse_double(fl[at + c], v[c])) return false;
    return true;
}

// An imported mesh: nodes (x, y, z) and panels of three or four node indices
// (0-based, a fourth of -1 for a triangle).
struct Imported {
    std::vector<double> xyz;
    std::vector<int> conn;
    std::string err;
    bool fail(const std::string& m) {
        err = m;
        return false;
    }
    void panel(int a, int b, int c, int d) { conn.insert(conn.end(), {a, b, c, d}); }
};

// GDF_Geometry::Read_Input_File / Generate_Nodes / Generate_Elements
// (GDF_Geo.cpp:12-103): a line of exactly three fields is a vertex; four
// consecutive vertices are a panel, a triangle when the fourth equals the
// third (GDF_Geo.cpp:39-41); every panel has its own nodes; scale 1.
bool read_gdf(std::istream& in, Imported& m) {
    std::vector<double> cur;
    std::string line;
    while (std::getline(in, line)) {
        const std::vector<std::string> fl = split_blank(line);
        if (fl.size() != 3) continue;
        double v[3];
        if (!parse_xyz(fl, 0, v)) return m.fail("non-numeric vertex line: " + line);
        cur.insert(cur.end(), v, v + 3);
        if (cur.size() < 12) continue;
        if (cur[9] == cur[6] && cur[10] == cur[7] && cur[11] == cur[8]) cur.resize(9);
        const int k = (int)(m.xyz.size() / 3), nv = (int)(cur.size() / 3);
        m.xyz.insert(m.xyz.end(), cur.begin(), cur.end());
        m.panel(k, k + 1, k + 2, nv == 4 ? k + 3 : -1);
        cur.clear();
    }
    return true;
}

// MAR_Geometry (MAR_Geo.cpp:12-96), the NEMOH mesh format: two-field lines
// (the symmetry header) are skipped; a four-field line whose first field is 0
// switches from nodes ("id x y z") to panels ("n1 n2 n3 n4", 1-based); a panel
// whose third and fourth fields are the same text is a triangle.  Nodes are
// numbered in file order, scale 1.
bool read_mar(std::istream& in, Imported& m) {
    bool panels = false;
    std::vector<long> ids;
    std::string line;
    while (std::getline(in, line)) {
        const std::vector<std::string> fl = split_blank(line);
        if (fl.size() != 4) continue;
        long id;
        if (!parse_int(fl[0], id)) return m.fail("non-numeric field: " + line);
        if (id == 0) {
            panels = true;
            continue;
        }
        if (panels) {
            long n[4];
            for (int c = 0; c < 4; ++c)
                if (!parse_int(fl[c], n[c])) return m.fail("non-numeric panel line: " + line);
            ids.insert(ids.end(), {n[0] - 1, n[1] - 1, n[2] - 1, fl[2] != fl[3] ? n[3] - 1 : -1});
        } else {
            double v[3];
            if (!parse_xyz(fl, 1, v)) return m.fail("non-numeric node line: " + line);
            m.xyz.insert(m.xyz.end(), v, v + 3);
        }
    }
    const long nn = (long)(m.xyz.size() / 3);
    for (size_t e = 0; e < ids.size(); e += 4) {
        for (int c = 0; c < 4; ++c)
            if ((c < 3 || ids[e + 3] != -1) && (ids[e + c] < 0 || ids[e + c] >= nn))
                return m.fail("panel " + std::to_string(e / 4) + " names a node that does not exist");
        m.panel((int)ids[e], (int)ids[e + 1], (int)ids[e + 2], (int)ids[e + 3]);
    }
    return true;
}

// STL_Geometry (STL_Geo.cpp:12-94), ASCII STL: a line starting "facet" opens a
// facet, its third to fifth lines ("vertex x y z") are the corners C1..C3;
// node positions are scaled by 100 (STL_Geo.cpp:62) and the triangle is
// stored as (C3, C2, C1), turning the normal from STL's outward convention to
// the solver's (STL_Geo.cpp:88-90).  Every facet has its own nodes.
bool read_stl(std::istream& in, Imported& m) {
    const double scale = 100.0;
    long count = -1000;  // lines since the last "facet"; none seen yet
    std::vector<double> cur;
    std::string line;
    while (std::getline(in, line)) {
        const std::vector<std::string> fl = split_blank(line);
        if (fl[0] == "facet") count = 0;
        if (count >= 2 && count <= 4) {
            double v[3];
            if (!parse_xyz(fl, 1, v)) return m.fail("bad vertex line: " + line);
            for (int c = 0; c < 3; ++c) cur.push_back(scale * v[c]);
            if (count == 4) {
                const int k = (int)(m.xyz.size() / 3);
                m.xyz.insert(m.xyz.end(), cur.begin(), cur.end());
                m.panel(k + 2, k + 1, k, -1);
                cur.clear();
            }
        }
        ++count;
    }
    return true;
}

bool has(const std::string& s, const char* t) { return s.find(t) != std::string::npos; }

// PNL_Geometry (PNL_Geo.cpp:17-129), the HAMS hull mesh format: marker lines
// ("Number of Panels", "Start/End Definition of Node Coordinates", "Start/End
// Definition of Node Relations") select the section; node lines are
// "id x y z", panel lines "id nv n1 n2 n3 [n4]" with 1-based node numbers.
// The symmetry flags of the count line are read and, as in the reference,
// not applied.  Scale 1.
bool read_pnl(std::istream& in, Imported& m) {
    int pos = 0;
    std::vector<long> ids;
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        if (has(line, "Number of Panels")) { pos = 1; continue; }
        if (has(line, "Start Definition of Node Coordinates")) { pos = 2; continue; }
        if (has(line, "End Definition of Node Coordinates")) { pos = 3; continue; }
        if (has(line, "Start Definition of Node Relations")) { pos = 4; continue; }
        if (has(line, "End Definition of Node Relations")) { pos = 5; continue; }
        const std::vector<std::string> fl = split_blank(line);
        if (pos == 1) {
            long c;
            if (fl.size() < 4) return m.fail("bad count line: " + line);
            for (int i = 0; i < 4; ++i)
                if (!parse_int(fl[i], c)) return m.fail("bad count line: " + line);
        } else if (pos == 2) {
            double v[3];
            if (!parse_xyz(fl, 1, v)) return m.fail("bad node line: " + line);
            m.xyz.insert(m.xyz.end(), v, v + 3);
        } else if (pos == 4) {
            long nv, n[4] = {0, 0, 0, 0};
            if (fl.size() < 5 || !parse_int(fl[1], nv)) return m.fail("bad panel line: " + line);
            const int take = nv == 4 ? 4 : 3;
            if ((int)fl.size() < 2 + take) return m.fail("bad panel line: " + line);
            for (int c = 0; c < take; ++c)
                if (!parse_int(fl[2 + c], n[c])) return m.fail("bad panel line: " + line);
            ids.insert(ids.end(), {n[0] - 1, n[1] - 1, n[2] - 1, take == 4 ? n[3] - 1 : -1});
        }
    }
    const long nn = (long)(m.xyz.size() / 3);
    for (size_t e = 0; e < ids.size(); e += 4) {
        for (int c = 0; c < 4; ++c)
            if ((c < 3 || ids[e + 3] != -1) && (ids[e + c] < 0 || ids[e + c] >= nn))
                return m.fail("panel " + std::to_string(e / 4) + " names a node that does not exist");
        m.panel((int)ids[e], (int)ids[e + 1], (int)ids[e + 2], (int)ids[e + 3]);
    }
    return true;
}

std::string g_import_err;

}  // namespace

extern "C" bem_status bem_read_mesh(const char* path, int format, int* n_nodes, double* nodes, int* n_elems,
                                    int* elems) {
    if (!path || !n_nodes || !n_elems) return BEM_ERR_ARG;
    const std::string p(path);
    if (format == BEM_MESH_AUTO) {
        // the console picks the reader by the extension it finds in the name
        // (BEMUser_Console.cpp:40-42); .pnl files go to PNL_Geometry
        format = has(p, ".gdf") ? BEM_MESH_GDF : has(p, ".mar") ? BEM_MESH_MAR
               : has(p, ".stl") ? BEM_MESH_STL : has(p, ".pnl") ? BEM_MESH_PNL : -1;
    }
    Imported m;
    std::ifstream f(path);
    bool ok;
    if (!f) ok = m.fail(p + " . A suitable mesh file was not found at this position.");
    else if (format == BEM_MESH_GDF) ok = read_gdf(f, m);
    else if (format == BEM_MESH_MAR) ok = read_mar(f, m);
    else if (format == BEM_MESH_STL) ok = read_stl(f, m);
    else if (format == BEM_MESH_PNL) ok = read_pnl(f, m);
    else ok = m.fail("unknown mesh format for " + p);
    if (!ok) {
        g_import_err = m.err;
        return BEM_ERR_ARG;
    }
    const int nn = (int)(m.xyz.size() / 3), ne = (int)(m.conn.size() / 4);
    if (nodes && elems) {
        if (*n_nodes < nn || *n_elems < ne) {
            g_import_err = "arrays too small";
            return BEM_ERR_ARG;
        }
        std::copy(m.xyz.begin(), m.xyz.end(), nodes);
        std::copy(m.conn.begin(), m.conn.end(), elems);
    }
    *n_nodes = nn;
    *n_elems = ne;
    return BEM_OK;
}

extern "C" const char* bem_read_mesh_error(void) { return g_import_err.c_str(); }
