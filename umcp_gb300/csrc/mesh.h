// Host-side mesh topology for the membrane-surface path: the .mesh text
// format of the reference (src/interpLib.C:1144-1600 loadLattice,
// src/write_structures.C:473-530 saveSurface), its orientation rule, the
// face enumeration of generatePlan (src/interpLib.C:5440-5560) and the
// synthetic-mesh generators used by tests and benchmarks.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace umcp {

struct Mesh {
  int nv = 0;
  double box[3][3] = {{1e10, 0, 0}, {0, 1e10, 0}, {0, 0, 1e10}};  // PBC_vec rows
  int fix_sense = 1;
  std::vector<double> r;          // 3*nv positions as read
  std::vector<int> valence;       // nv
  std::vector<int> nbr_off;       // nv+1 offsets into nbr
  std::vector<int> nbr;           // neighbour ids, oriented order after orient()
  std::vector<int> tri;           // explicit triangles from an "ntri" block (3 per)

  int nbr_of(int i, int e) const { return nbr[nbr_off[i] + e]; }
  int find_nbr(int i, int j) const;  // index e with nbr_of(i,e)==j, or -1
};

// One face of the limit surface: lowest-index corner i, and the one-ring
// control points in the reference's point_list order (src/interpLib.C:5537-5553).
struct Face {
  int i, j, k;          // corners; j = edges[e], k = edges[e+1] of i
  int valence;          // valence of i (6 => regular)
  int ncp;              // valence + 6
  int cp[13];           // control-point vertex ids
  int8_t img[13][3];    // lattice-image shift of each control point relative to cp[0]
};

// Parse a .mesh file. Returns "" on success, else an error message.
std::string read_mesh(const std::string &path, Mesh *m);
// Write the .mesh format (full precision positions).
std::string write_mesh(const std::string &path, const Mesh &m);

// Orient every vertex's neighbour ring following the reference's rule
// (triangle senses propagated from triangle 0, src/interpLib.C:1780-2030).
std::string orient(Mesh *m);

// Enumerate faces in generatePlan order; regular faces first list, irregular second.
std::string enumerate_faces(const Mesh &m, std::vector<Face> *regular, std::vector<Face> *irregular);

// Minimum-image lattice shift of dr (greedy search of src/mutil.C:541-599).
// Squared length below which min_image_shift finds no shift for this box.
double min_image_free_r2(const double box[3][3]);
// Lattice shift (each -1..1, repeated while it shortens) taking dr to its
// minimum image; vectors shorter than sqrt(free_r2) return no shift at once.
void min_image_shift(const double dr[3], const double box[3][3], int shift[3], double free_r2 = 0.0);

// Synthetic meshes. Vesicle: icosahedron Loop-subdivided `level` times (original
// 12 vertices first), projected to radius R, radial Gaussian noise sigma (Philox
// keyed by seed and vertex id), box 3R. Planar: nx*ny triangular lattice of
// spacing a with a q^-4 height spectrum of variance kT/(kc_kT * Lx*Ly*q^4).
void generate_icosphere(int level, double R, double sigma, uint64_t seed, Mesh *m);
void generate_planar(int nx, int ny, double a, double kc_kT, uint64_t seed, Mesh *m);

}  // namespace umcp
