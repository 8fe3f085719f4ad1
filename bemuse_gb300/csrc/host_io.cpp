// host_io.cpp -- result files in the WAMIT formats the reference writes
// (Hydrodynamic_Solver_IO.cpp:430-646): .1 added mass / damping, .2 Haskind
// excitation, .2fk Froude-Krylov, .2sc scattering, .4 RAO, .hst hydrostatic
// stiffness, .mmx mass matrix.  Host only.
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
