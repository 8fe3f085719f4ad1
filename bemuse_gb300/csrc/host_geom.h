// host_geom.h -- host-side mesh generators and panel geometry.
#pragma once
#include <string>
#include <vector>
#include "bem_internal.h"

namespace bem {

struct MeshView {
    int n_nodes;
    const double* nodes;
    int n_elems;
    const int* elems;
    int n_comp;
    const int* comp_first;
    const double* comp_origin;
};

// One flat panel: vertices (global), centroid, frame rows ex|ey|ez (ez = normal),
// area, and its quadrature nodes (position, weight x Jacobian, unit normal).
struct PanelGeom {
    int nv;
    double v[12];
    double c[3];
    double e[9];
    double area;
    int nq;
    double qp[12];
    double qw[4];
    double qn[12];
};

bool build_geometry(const MeshView& m, std::vector<PanelGeom>& body, std::vector<PanelGeom>& mirror,
                    std::string& err);
void rankine_record(const PanelGeom& p, double* rec);
void collocation_points(const std::vector<PanelGeom>& body, std::vector<double>& xr);
void cylinder_sizes(int NA, int NR, int NV, int NRFS, int* nn, int* ne, int* nna, int* nea);
void cylinder_mesh(double R, double draft, int NA, int NR, int NV, int NRFS, bool cosine, double* nodes, int* elems,
                   double* aux_nodes, int* aux_elems);
void barge_sizes(int NX, int NY, int NZ, int* nn, int* ne, int* nna, int* nea);
void barge_mesh(double L, double W, double D, int NX, int NY, int NZ, bool cosine, double* nodes, int* elems,
                double* aux_nodes, int* aux_elems);
void wing_sizes(int nc, int ns, int* nn, int* ne);
void wing_mesh(double chord, double span, double t, int nc, int ns, bool cosine, double* nodes, int* elems);
void wing_wake(double chord, double span, int nc, int ns, double length, double* quads, int* te_up, int* te_lo);
void mass_and_stiffness(const std::vector<PanelGeom>& body, const std::vector<PanelGeom>* aux, double rho, double g,
                        double mass, const double* cog, const double* gyr, double* M, double* C, double* vc);

}  // namespace bem
