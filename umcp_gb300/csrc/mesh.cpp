// Mesh format, orientation, face enumeration and synthetic generators.
// See mesh.h for the reference functions each part follows.
#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <string>

#include "philox.h"

namespace umcp {

int Mesh::find_nbr(int i, int j) const {
  for (int e = 0; e < valence[i]; ++e)
    if (nbr_of(i, e) == j) return e;
  return -1;
}

// ---------------------------------------------------------------- I/O

static bool starts_with_nocase(const char *s, const char *p) {
  for (; *p; ++s, ++p)
    if (tolower((unsigned char)*s) != tolower((unsigned char)*p)) return false;
  return true;
}

std::string read_mesh(const std::string &path, Mesh *m) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return "cannot open mesh file '" + path + "'";
  *m = Mesh();
  std::vector<std::string> lines;
  {
    char buf[1 << 16];
    while (fgets(buf, sizeof buf, f)) lines.emplace_back(buf);
  }
  fclose(f);
  size_t ln = 0;
  auto next = [&](std::string *out) -> bool {
    if (ln >= lines.size()) return false;
    *out = lines[ln++];
    return true;
  };
  std::string line;
  if (!next(&line)) return "empty mesh file";
  bool vec3 = starts_with_nocase(line.c_str(), "3D");
  int nvec = vec3 ? 3 : 2;
  for (int d = 0; d < nvec; ++d) {
    if (!next(&line)) return "truncated box header";
    if (sscanf(line.c_str(), "%lf %lf %lf", &m->box[d][0], &m->box[d][1], &m->box[d][2]) != 3)
      return "bad box vector line";
  }
  if (!vec3) { m->box[2][0] = 0; m->box[2][1] = 0; m->box[2][2] = 1e6; }
  // optional "sense N"
  if (ln < lines.size() && starts_with_nocase(lines[ln].c_str(), "sense")) {
    sscanf(lines[ln].c_str() + 5, "%d", &m->fix_sense);
    ++ln;
  }
  std::vector<std::vector<int>> nb;
  bool have_tri = false;
  int ntri = 0;
  while (next(&line)) {
    const char *s = line.c_str();
    while (*s == ' ' || *s == '\t') ++s;
    if (starts_with_nocase(s, "ntri")) { have_tri = true; sscanf(s + 4, "%d", &ntri); break; }
    int id, val;
    double x, y, z;
    const char *body = s;
    int skip_doubles = 0;
    if (*s == 'P') { body = s + 1; skip_doubles = 15; }
    else if (*s == 'Q') { body = s + 1; }
    // whitespace-separated fields: id x y z [15 doubles after 'P'] valence ring...
    const char *q = body;
    char *end = nullptr;
    auto int_field = [&](int *out) {
      const long v = strtol(q, &end, 10);
      if (end == q) return false;
      q = end;
      *out = (int)v;
      return true;
    };
    auto dbl_field = [&](double *out) {
      const double v = strtod(q, &end);
      if (end == q) return false;
      q = end;
      *out = v;
      return true;
    };
    if (!int_field(&id) || !dbl_field(&x) || !dbl_field(&y) || !dbl_field(&z)) continue;
    bool ok = true;
    for (int k = 0; k < skip_doubles && ok; ++k) { double t; ok = dbl_field(&t); }
    if (!ok || !int_field(&val)) continue;
    if (val < 5 || val > 7) return "vertex valence must be between 5 and 7";
    std::vector<int> ring;
    int n;
    while ((int)ring.size() < val && int_field(&n)) ring.push_back(n);
    if ((int)ring.size() != val) return "vertex line has fewer neighbours than its valence";
    m->r.push_back(x); m->r.push_back(y); m->r.push_back(z);
    m->valence.push_back(val);
    nb.push_back(ring);
  }
  m->nv = (int)m->valence.size();
  if (m->nv == 0) return "mesh has no vertices";
  m->nbr_off.assign(m->nv + 1, 0);
  for (int i = 0; i < m->nv; ++i) m->nbr_off[i + 1] = m->nbr_off[i] + m->valence[i];
  m->nbr.resize(m->nbr_off[m->nv]);
  for (int i = 0; i < m->nv; ++i)
    for (int e = 0; e < m->valence[i]; ++e) {
      int j = nb[i][e];
      if (j < 0 || j >= m->nv || j == i) return "neighbour index out of range";
      m->nbr[m->nbr_off[i] + e] = j;
    }
  for (int i = 0; i < m->nv; ++i)
    for (int e = 0; e < m->valence[i]; ++e)
      if (m->find_nbr(m->nbr_of(i, e), i) < 0) return "neighbour lists are not symmetric";
  if (have_tri) {
    for (int t = 0; t < ntri; ++t) {
      if (!next(&line)) return "truncated triangle block";
      int a, b, c;
      if (sscanf(line.c_str(), "%d %d %d", &a, &b, &c) != 3) return "bad triangle line";
      m->tri.push_back(a); m->tri.push_back(b); m->tri.push_back(c);
    }
  }
  return "";
}

std::string write_mesh(const std::string &path, const Mesh &m) {
  FILE *f = fopen(path.c_str(), "w");
  if (!f) return "cannot write mesh file '" + path + "'";
  bool planar = (m.box[2][0] == 0 && m.box[2][1] == 0 && m.box[2][2] == 1e6);
  if (planar) {
    fprintf(f, "2D umcp-gb300 mesh\n");
    for (int d = 0; d < 2; ++d) fprintf(f, "%.17g %.17g %.17g\n", m.box[d][0], m.box[d][1], m.box[d][2]);
  } else {
    fprintf(f, "3D umcp-gb300 mesh\n");
    for (int d = 0; d < 3; ++d) fprintf(f, "%.17g %.17g %.17g\n", m.box[d][0], m.box[d][1], m.box[d][2]);
  }
  if (m.fix_sense != 1) fprintf(f, "sense %d\n", m.fix_sense);
  for (int i = 0; i < m.nv; ++i) {
    fprintf(f, "%d %.17g %.17g %.17g %d", i, m.r[3 * i], m.r[3 * i + 1], m.r[3 * i + 2], m.valence[i]);
    for (int e = 0; e < m.valence[i]; ++e) fprintf(f, " %d", m.nbr_of(i, e));
    fprintf(f, "\n");
  }
  fclose(f);
  return "";
}

// ---------------------------------------------------------------- orientation

namespace {
struct Tri { int id[3]; int sense; };
struct Edge { int v0, v1; int face[3]; int code[3]; };
}  // namespace

// Relative sense of two triangles sharing an edge: with ids sorted a<b<c the
// edge codes are (a,b)=2, (a,c)=1, (b,c)=0, and a consistent orientation
// traverses the shared edge in opposite directions (src/interpLib.C:110-121).
static int compare_sense(int c1, int c2) { return ((c1 == 1) != (c2 == 1)) ? 1 : -1; }

std::string orient(Mesh *m) {
  const int nv = m->nv;
  std::vector<Tri> tris;
  // Triangle discovery order of constructTriangles (src/interpLib.C:7222-7290),
  // which the reference re-runs on the file-order rings before it assigns
  // senses (src/interpLib.C:1784-1790); an "ntri" block does not change it.
  {
    for (int i = 0; i < nv; ++i)
      for (int vi = 0; vi < m->valence[i]; ++vi) {
        int j = m->nbr_of(i, vi);
        if (j < i) continue;
        for (int vj = 0; vj < m->valence[j]; ++vj) {
          int k = m->nbr_of(j, vj);
          if (k == i || k < j) continue;
          if (m->find_nbr(k, i) >= 0) tris.push_back({{i, j, k}, 0});
        }
      }
  }
  if (tris.empty()) return "mesh has no triangles";
  // Edges with the faces on each side, in creation order. The edge (a, b),
  // a < b, is found through slot e of a's ring (eslot[nbr_off[a] + e]).
  std::vector<int> eslot(m->nbr.size(), -1);
  std::vector<Edge> edges;
  for (size_t t = 0; t < tris.size(); ++t) {
    const int *s = tris[t].id;
    int pairs[3][2] = {{s[0], s[1]}, {s[0], s[2]}, {s[1], s[2]}};
    int codes[3] = {2, 1, 0};
    for (int p = 0; p < 3; ++p) {
      const int a = pairs[p][0], b = pairs[p][1];
      int &slot = eslot[m->nbr_off[a] + m->find_nbr(a, b)];
      if (slot < 0) {
        slot = (int)edges.size();
        edges.push_back(Edge{a, b, {(int)t, -1, -1}, {codes[p], -1, -1}});
      } else {
        Edge &e = edges[slot];
        int k = (e.face[1] == -1) ? 1 : 2;
        e.face[k] = (int)t;
        e.code[k] = codes[p];
      }
    }
  }
  // Senses from triangle 0 (src/interpLib.C:1790-1825), across the edges'
  // first two faces. On a connected orientable surface the senses are fixed
  // by triangle 0's, so one breadth-first pass gives what repeated sweeps
  // over the edge list give; every such edge is checked for consistency.
  {
    std::vector<std::vector<int>> tedges(tris.size());
    for (size_t e = 0; e < edges.size(); ++e)
      if (edges[e].face[0] >= 0 && edges[e].face[1] >= 0) {
        tedges[edges[e].face[0]].push_back((int)e);
        tedges[edges[e].face[1]].push_back((int)e);
      }
    tris[0].sense = m->fix_sense;
    std::vector<int> queue(1, 0);
    for (size_t h = 0; h < queue.size(); ++h) {
      const int t = queue[h];
      for (int e : tedges[t]) {
        const Edge &E = edges[e];
        const int u = E.face[0] == t ? E.face[1] : E.face[0];
        const int want = tris[t].sense * compare_sense(E.code[0], E.code[1]);
        if (!tris[u].sense) {
          tris[u].sense = want;
          queue.push_back(u);
        } else if (tris[u].sense != want) {
          return "surface is not orientable";
        }
      }
    }
  }
  // Oriented successor map: for an oriented triangle (a,b,c), around vertex a
  // the ring steps from c to b (the reference's sorted rings list edges[e],
  // edges[e+1] such that (i, edges[e+1], edges[e]) is positively oriented).
  // Vertex a's pairs (c -> b) live in slots nbr_off[a] .. (at most its valence).
  std::vector<int> skey(m->nbr.size()), sval(m->nbr.size()), scount(nv, 0);
  auto put = [&](int a, int key, int val) -> bool {
    const int o = m->nbr_off[a];
    for (int q = 0; q < scount[a]; ++q)
      if (skey[o + q] == key) { sval[o + q] = val; return true; }
    if (scount[a] >= m->valence[a]) return false;
    skey[o + scount[a]] = key;
    sval[o + scount[a]] = val;
    ++scount[a];
    return true;
  };
  auto get = [&](int a, int key) -> int {
    const int o = m->nbr_off[a];
    for (int q = 0; q < scount[a]; ++q)
      if (skey[o + q] == key) return sval[o + q];
    return -1;
  };
  for (const Tri &t : tris) {
    if (!t.sense) return "mesh has triangles not reachable from triangle 0";
    int a = t.id[0], b = t.id[1], c = t.id[2];
    if (t.sense < 0) std::swap(b, c);  // oriented cycle a->b->c
    if (!put(a, c, b) || !put(b, a, c) || !put(c, b, a)) return "a vertex lies on more triangles than its valence";
  }
  for (int i = 0; i < nv; ++i) {
    int val = m->valence[i];
    std::vector<int> ring;
    int cur = m->nbr_of(i, 0);
    ring.push_back(cur);
    for (int s = 1; s < val; ++s) {
      const int nx = get(i, cur);
      if (nx < 0) return "vertex " + std::to_string(i) + " has an open or broken ring";
      cur = nx;
      ring.push_back(cur);
    }
    const int nx = get(i, cur);
    if (nx < 0 || nx != ring[0]) return "vertex " + std::to_string(i) + " ring does not close";
    for (int e = 0; e < val; ++e) m->nbr[m->nbr_off[i] + e] = ring[e];
  }
  return "";
}

// ---------------------------------------------------------------- faces

// Squared length under which no lattice shift can shorten a vector: a
// shift t shortens dr only if |dr| > |t| / 2, so a quarter of the shortest
// nonzero combination of the box vectors (less a relative margin).
double min_image_free_r2(const double box[3][3]) {
  double best = 0.0;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        if (!dx && !dy && !dz) continue;
        double t2 = 0.0;
        for (int c = 0; c < 3; ++c) {
          const double t = dx * box[0][c] + dy * box[1][c] + dz * box[2][c];
          t2 += t * t;
        }
        if (best == 0.0 || t2 < best) best = t2;
      }
  return 0.25 * best * (1.0 - 1e-9);
}

void min_image_shift(const double dr[3], const double box[3][3], int shift[3], double free_r2) {
  shift[0] = shift[1] = shift[2] = 0;
  if (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2] < free_r2) return;
  double tr[3] = {dr[0], dr[1], dr[2]};
  bool done = false;
  while (!done) {
    done = true;
    double r2 = tr[0] * tr[0] + tr[1] * tr[1] + tr[2] * tr[2];
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          double add[3];
          for (int c = 0; c < 3; ++c) add[c] = dx * box[0][c] + dy * box[1][c] + dz * box[2][c];
          double t[3] = {tr[0] + add[0], tr[1] + add[1], tr[2] + add[2]};
          double nr2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
          if (!(nr2 >= r2 - 1e-7)) {
            tr[0] = t[0]; tr[1] = t[1]; tr[2] = t[2];
            r2 = nr2;
            shift[0] += dx; shift[1] += dy; shift[2] += dz;
            done = false;
          }
        }
  }
}

std::string enumerate_faces(const Mesh &m, std::vector<Face> *regular, std::vector<Face> *irregular) {
  regular->clear();
  irregular->clear();
  const double free_r2 = min_image_free_r2(m.box);
  for (int i = 0; i < m.nv; ++i) {
    int val = m.valence[i];
    for (int e = 0; e < val; ++e) {
      int ep1 = (e + 1) % val;
      int j = m.nbr_of(i, e), k = m.nbr_of(i, ep1);
      if (j < i || k < i) continue;
      int valj = m.valence[j], valk = m.valence[k];
      if (valj != 6 || valk != 6)
        return "illegal mesh: a face touches two irregular vertices or its irregular vertex is not its lowest index (vertices " +
               std::to_string(i) + "," + std::to_string(j) + "," + std::to_string(k) + ")";
      int ej = m.find_nbr(j, i), ek = m.find_nbr(k, i);
      auto wrap = [](int x, int n) { return ((x % n) + n) % n; };
      Face f{};
      f.i = i; f.j = j; f.k = k;
      f.valence = val;
      f.ncp = val + 6;
      f.cp[0] = i;
      f.cp[1] = k;
      f.cp[2] = j;
      for (int q = 1; q <= val - 2; ++q) f.cp[2 + q] = m.nbr_of(i, wrap(e - q, val));
      f.cp[val + 1] = m.nbr_of(k, wrap(ek - 2, valk));
      f.cp[val + 2] = m.nbr_of(k, wrap(ek + 3, valk));
      f.cp[val + 3] = m.nbr_of(k, wrap(ek + 2, valk));
      f.cp[val + 4] = m.nbr_of(j, wrap(ej + 3, valj));
      f.cp[val + 5] = m.nbr_of(j, wrap(ej + 2, valj));
      const double *r0 = &m.r[3 * i];
      for (int p = 0; p < f.ncp; ++p) {
        const double *r1 = &m.r[3 * f.cp[p]];
        double dr[3] = {r1[0] - r0[0], r1[1] - r0[1], r1[2] - r0[2]};
        int s[3];
        min_image_shift(dr, m.box, s, free_r2);
        for (int c = 0; c < 3; ++c) {
          if (s[c] < -1 || s[c] > 1) return "control point more than one box away from its face";
          f.img[p][c] = (int8_t)s[c];
        }
      }
      (val == 6 ? regular : irregular)->push_back(f);
    }
  }
  return "";
}

// ---------------------------------------------------------------- generators

static void normal_pair(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, double *n0, double *n1) {
  philox_out o = philox4x32_10(c0, c1, c2, 0x6d657368u, (uint32_t)seed, (uint32_t)(seed >> 32));
  double u1 = philox_u53(o.v[0], o.v[1]), u2 = philox_u53(o.v[2], o.v[3]);
  double rad = std::sqrt(-2.0 * std::log(u1));
  *n0 = rad * std::cos(2.0 * M_PI * u2);
  *n1 = rad * std::sin(2.0 * M_PI * u2);
}

// Build CCW neighbour rings from oriented triangles (each listed a->b->c).
static void rings_from_triangles(int nv, const std::vector<int> &tris, Mesh *m) {
  std::vector<std::map<int, int>> next(nv);  // around a: b -> c  (CCW)
  for (size_t t = 0; t < tris.size() / 3; ++t) {
    int a = tris[3 * t], b = tris[3 * t + 1], c = tris[3 * t + 2];
    next[a][b] = c; next[b][c] = a; next[c][a] = b;
  }
  m->valence.assign(nv, 0);
  m->nbr_off.assign(nv + 1, 0);
  m->nbr.clear();
  for (int v = 0; v < nv; ++v) {
    int start = next[v].begin()->first;  // smallest-id neighbour first
    int cur = start;
    do {
      m->nbr.push_back(cur);
      cur = next[v][cur];
    } while (cur != start);
    m->valence[v] = (int)(m->nbr.size() - m->nbr_off[v]);
    m->nbr_off[v + 1] = (int)m->nbr.size();
  }
}

void generate_icosphere(int level, double R, double sigma, uint64_t seed, Mesh *m) {
  *m = Mesh();
  const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
  std::vector<double> p = {0, 1, phi, 0, -1, phi, 0, 1, -phi, 0, -1, -phi, 1, phi, 0, -1, phi, 0,
                           1, -phi, 0, -1, -phi, 0, phi, 0, 1, -phi, 0, 1, phi, 0, -1, -phi, 0, -1};
  for (size_t v = 0; v < 12; ++v) {
    double n = std::sqrt(p[3 * v] * p[3 * v] + p[3 * v + 1] * p[3 * v + 1] + p[3 * v + 2] * p[3 * v + 2]);
    for (int c = 0; c < 3; ++c) p[3 * v + c] /= n;
  }
  // The 20 faces: vertex triples at the minimal pairwise distance, oriented outward.
  std::vector<int> tris;
  auto d2 = [&](int a, int b) {
    double s = 0;
    for (int c = 0; c < 3; ++c) s += (p[3 * a + c] - p[3 * b + c]) * (p[3 * a + c] - p[3 * b + c]);
    return s;
  };
  double emin = 1e9;
  for (int a = 0; a < 12; ++a)
    for (int b = a + 1; b < 12; ++b) emin = std::min(emin, d2(a, b));
  for (int a = 0; a < 12; ++a)
    for (int b = a + 1; b < 12; ++b)
      for (int c = b + 1; c < 12; ++c) {
        if (d2(a, b) > emin * 1.01 || d2(a, c) > emin * 1.01 || d2(b, c) > emin * 1.01) continue;
        double u[3], w[3], cr[3];
        for (int q = 0; q < 3; ++q) { u[q] = p[3 * b + q] - p[3 * a + q]; w[q] = p[3 * c + q] - p[3 * a + q]; }
        cr[0] = u[1] * w[2] - u[2] * w[1]; cr[1] = u[2] * w[0] - u[0] * w[2]; cr[2] = u[0] * w[1] - u[1] * w[0];
        double dot = cr[0] * p[3 * a] + cr[1] * p[3 * a + 1] + cr[2] * p[3 * a + 2];
        if (dot > 0) { tris.push_back(a); tris.push_back(b); tris.push_back(c); }
        else { tris.push_back(a); tris.push_back(c); tris.push_back(b); }
      }
  // Loop topology: one new vertex per edge, appended after the existing ones.
  for (int l = 0; l < level; ++l) {
    std::map<std::pair<int, int>, int> mid;
    std::vector<int> nt;
    auto midpoint = [&](int a, int b) {
      auto key = std::make_pair(std::min(a, b), std::max(a, b));
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      int id = (int)(p.size() / 3);
      double q[3], n = 0;
      for (int c = 0; c < 3; ++c) { q[c] = 0.5 * (p[3 * a + c] + p[3 * b + c]); n += q[c] * q[c]; }
      n = std::sqrt(n);
      for (int c = 0; c < 3; ++c) p.push_back(q[c] / n);
      mid[key] = id;
      return id;
    };
    for (size_t t = 0; t < tris.size() / 3; ++t) {
      int a = tris[3 * t], b = tris[3 * t + 1], c = tris[3 * t + 2];
      int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      int add[12] = {a, ab, ca, ab, b, bc, ca, bc, c, ab, bc, ca};
      nt.insert(nt.end(), add, add + 12);
    }
    tris.swap(nt);
  }
  int nv = (int)(p.size() / 3);
  m->nv = nv;
  m->r.resize(3 * nv);
  for (int v = 0; v < nv; ++v) {
    double n0, n1;
    normal_pair(seed, (uint32_t)v, 0u, 0u, &n0, &n1);
    double rad = R + sigma * n0;
    for (int c = 0; c < 3; ++c) m->r[3 * v + c] = rad * p[3 * v + c];
  }
  for (int d = 0; d < 3; ++d)
    for (int c = 0; c < 3; ++c) m->box[d][c] = (d == c) ? 3.0 * R : 0.0;
  rings_from_triangles(nv, tris, m);
}

void generate_planar(int nx, int ny, double a, double kc_kT, uint64_t seed, Mesh *m) {
  *m = Mesh();
  if (ny % 2) ny += 1;  // the row offset pattern closes only for an even row count
  const double h = a * std::sqrt(3.0) / 2.0;
  const double Lx = nx * a, Ly = ny * h;
  int nv = nx * ny;
  m->nv = nv;
  m->r.resize(3 * nv);
  auto id = [&](int i, int j) { return ((j % ny + ny) % ny) * nx + ((i % nx + nx) % nx); };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      int v = id(i, j);
      m->r[3 * v] = a * (i + 0.5 * (j & 1));
      m->r[3 * v + 1] = h * j;
      m->r[3 * v + 2] = 0.0;
    }
  // q^-4 height spectrum: h = sum_q A_q cos(q.r + phi_q) over the half plane
  // of lattice-commensurate q with 0 < |q| <= pi/a, Var(A_q) = 1/(kc_kT Lx Ly q^4).
  const double qmax = M_PI / a;
  int mmax = (int)std::floor(qmax * Lx / (2 * M_PI)), nmax = (int)std::floor(qmax * Ly / (2 * M_PI));
  // Separable evaluation: with x = a (i + s/2) (s = row parity) and y = h j,
  //   z(i,j) = Re sum_n e^{2 pi i n j / ny} F_n(i, s),
  //   F_n(i, s) = sum_m A_mn e^{i phi_mn} e^{2 pi i m (i + s/2) / nx}.
  std::vector<std::vector<std::pair<int, std::complex<double>>>> rows(nmax + 1);
  for (int nn = 0; nn <= nmax; ++nn)
    for (int mm = -mmax; mm <= mmax; ++mm) {
      if (nn == 0 && mm <= 0) continue;
      double kx = 2 * M_PI * mm / Lx, ky = 2 * M_PI * nn / Ly;
      double q2 = kx * kx + ky * ky;
      if (q2 > qmax * qmax) continue;
      double g0, g1;
      normal_pair(seed, (uint32_t)(mm + 65536), (uint32_t)nn, 1u, &g0, &g1);
      double sd = std::sqrt(1.0 / (kc_kT * Lx * Ly * q2 * q2));
      double amp = sd * g0;
      double ph = M_PI * (1.0 + std::erf(g1 / std::sqrt(2.0)));  // uniform phase in [0, 2pi)
      rows[nn].push_back({mm, std::polar(amp, ph)});
    }
  std::vector<std::complex<double>> F((size_t)2 * nx);
  std::vector<double> z((size_t)nv, 0.0);
  for (int nn = 0; nn <= nmax; ++nn) {
    if (rows[nn].empty()) continue;
    for (int sp = 0; sp < 2; ++sp)
      for (int i = 0; i < nx; ++i) {
        std::complex<double> acc = 0;
        for (const auto &mc : rows[nn]) acc += mc.second * std::polar(1.0, 2 * M_PI * mc.first * (i + 0.5 * sp) / nx);
        F[(size_t)sp * nx + i] = acc;
      }
    for (int j = 0; j < ny; ++j) {
      std::complex<double> e = std::polar(1.0, 2 * M_PI * nn * (double)j / ny);
      const std::complex<double> *Fr = &F[(size_t)(j & 1) * nx];
      for (int i = 0; i < nx; ++i) z[id(i, j)] += (Fr[i] * e).real();
    }
  }
  for (int v = 0; v < nv; ++v) m->r[3 * v + 2] = z[v];
  m->box[0][0] = Lx; m->box[0][1] = 0; m->box[0][2] = 0;
  m->box[1][0] = 0; m->box[1][1] = Ly; m->box[1][2] = 0;
  m->box[2][0] = 0; m->box[2][1] = 0; m->box[2][2] = 1e6;
  std::vector<int> tris;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      int v = id(i, j);
      int right = id(i + 1, j);
      int ur = (j & 1) ? id(i + 1, j + 1) : id(i, j + 1);
      int ul = (j & 1) ? id(i, j + 1) : id(i - 1, j + 1);
      tris.push_back(v); tris.push_back(right); tris.push_back(ur);
      tris.push_back(v); tris.push_back(ur); tris.push_back(ul);
    }
  rings_from_triangles(nv, tris, m);
}

}  // namespace umcp
