// Host-side plan builder for the limit-surface energy: the per-point basis rows
// of surface::generatePlan (src/interpLib.C:4998-6669), the irregular-vertex
// quadrature of src/gauss.C, and the reference state of surface::setg0
// (src/interpLib.C:2969-3390). Everything here runs once per mesh.
#pragma once
#include <string>
#include <vector>

#include "mesh.h"

namespace umcp {

constexpr int kRegPts = 15;   // G_Q_P_15 rule, src/interpLib.C:5336-5375
constexpr int kIrrPts = 16;   // n_u_gauss * n_v_finite = 4 * 4, src/interpLib.C:50-51
constexpr int kKinds = 6;     // basis rows: w, u, v, uu, uv, vv
constexpr int kMaxCp = 13;    // valence 7 + 6

// Basis rows of one patch type: row[(kind*npt + pt)*ncp + cp], point weights.
struct PatchBasis {
  int valence = 6, ncp = 12, npt = kRegPts;
  std::vector<double> row;
  std::vector<double> weight;
  std::vector<double> u, v;  // quadrature point in face coordinates
  double at(int kind, int pt, int cp) const { return row[((size_t)kind * npt + pt) * ncp + cp]; }
};

// Lipid library entry and the leaflet assignment of a bilayer composition.
struct Lipid { std::string name; double c0, apl, outer_parts, inner_parts; };

struct Plan {
  PatchBasis regular;
  PatchBasis irregular[8];           // indexed by valence (5 and 7 used)
  std::vector<Face> reg_faces, irr_faces;
  std::vector<double> reg_g0, reg_RuRv0;   // [face*15 + pt]
  std::vector<double> irr_g0, irr_RuRv0;   // [face*16 + pt]
  std::vector<double> ref_r;               // the state g0 and RuRv0 were taken at (3*nv)
  // Leaflet compositions: areas (A^2) per lipid type, [face*ntypes + x].
  int ntypes = 1;
  std::vector<Lipid> lipids;
  std::vector<double> reg_outer, reg_inner, irr_outer, irr_inner;
};

// The 12 quartic box-spline basis functions of a regular Loop patch and their
// first and second derivatives at (u,v), in the reference's control-point
// order (ceff_map, src/interpLib.C:6012): out[kind][cp].
void box_spline_rows(double u, double v, double out[kKinds][12]);
// The values alone (the w row of box_spline_rows), out[cp].
void box_spline_values(double u, double v, double out[12]);

// Gauss nodes/weights for the singular weights of an irregular patch
// (src/gauss.C get_v_pts / get_u_pts): n points, eigenvalue parameter k.
void irregular_gauss_v(int n, double k, double *x, double *w);
void irregular_gauss_u(int n, double k, double v, double *x, double *w);

// Subdivision eigenvalue parameter k for a valence (src/interpLib.C:5560-5570).
double irregular_k(int valence);

void build_regular_basis(PatchBasis *b);
std::string build_irregular_basis(int valence, PatchBasis *b);

// The irregular patch's map at (u,v) (irr_kernel::get_map,
// src/irr_kernel.C:474-541): moves (u,v) into the coordinates of the
// sub-triangle of its domain ring, returns the derivative scale of that move,
// and cmap[y][x] = (Atot A^(domain-1))[pcycle[y]][x], the weights of control
// point x in box spline y of the sub-triangle. Powers of A are cached.
class IrregularMap {
 public:
  explicit IrregularMap(int valence);
  void at(double *u, double *v, double *scale, double cmap[12][kMaxCp]);

 private:
  const std::vector<double> &power(int e);
  int val_, n_;
  std::vector<double> atot_;
  std::vector<std::vector<double>> powers_;
};

// Loop subdivision of a regular 12-point patch into its four children
// (fast_sub6_0..3, src/fast_mm.C): child k's control point x is
// sum_y S[k][x][y] P[y], in the reference's child numbering and point order.
void subdivision_stencils(double S[4][12][12]);

// Limit-surface point at (u,v) of a face as weights of the face's control
// points (surface::get_pt_coeffs, src/uv_map.C:14-195): coef[x] for cp[x].
// maps[valence] serves irregular faces. Returns the number of weights.
int limit_point_coeffs(const Face &f, double u, double v, IrregularMap *maps[8], double *coef);

// The value rows with the u and v derivative rows (surface::evaluateRNRM,
// src/interpLib.C:7936); at an extraordinary vertex itself the derivatives
// are NaN, as the reference leaves the normal there.
int limit_point_rows(const Face &f, double u, double v, IrregularMap *maps[8], double *w, double *du, double *dv);

// Effective mass of the limit surface (getSparseEffectiveMass,
// src/modes.C:1735-1740): M = sum over mass points k of m c_k c_k^T, with the
// (plim+1)(plim+2)/2 points per face and the mass per point of src/hd.C:417-452.
// Every mass point of a face is a combination of the face's own control
// points with weights that depend on the patch type only, so M is the sum
// over faces of one block per patch type placed at the face's control points.
struct MassPoints {
  double area0 = 0, mass_per_point = 0;
  long long points = 0;
};
MassPoints mass_points(const Plan &p, double mass_scale, int plim);
// B[a*ncp + b] = m sum over a face's points of c_a c_b, for the patch type of
// a corner of this valence (6: regular, ncp 12).
void face_mass_block(int valence, int ncp, int plim, double m, double *B);

// Parses the lipid directives of an input file ("lipid library NAME APL c0",
// "lipid outer NAME parts", "lipid inner NAME parts"; src/lipid_composition.C:47-300).
std::string parse_lipids(const std::string &text, std::vector<Lipid> *lipids);

// Full plan for an oriented mesh; reference state from the mesh positions.
std::string build_plan(const Mesh &m, const std::vector<Lipid> &lipids, Plan *p);

// setg0: g0 and RuRv0 at every point of the state r (3*nv doubles, no box
// scaling) and the whole-lipid leaflet fill of each face.
void set_reference_state(const Mesh &m, const double *r, Plan *p);

// Completed-square form of the lipid bending term of one face:
//   sum_x 0.25*kc*w*[out_x (H-c0_x)^2 + in_x (-H-c0_x)^2] = 0.25*kc*w*(P2 (H-Hbar)^2 + Pres)
void composition_coeffs(const double *outer, const double *inner, const std::vector<Lipid> &lipids,
                        double *P2, double *Hbar, double *Pres);

}  // namespace umcp
