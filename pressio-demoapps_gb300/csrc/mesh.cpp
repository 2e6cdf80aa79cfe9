// Mesh files (the reference's text format and a binary format of this
// library), native full-mesh and sample-mesh generators, and the
// inner/near-boundary row classification.
//
// The generators reproduce the connectivity rules of the reference's
// meshing scripts (meshing_scripts/_impl/one_dim_mesh.py:41-146,
// natural_order_mesh_2d.py:78-258, natural_order_mesh_3d.py:96-225 and
// create_sample_mesh.py:28-137) so that files and in-memory graphs are
// identical to what the scripts produce; the branch structure of each rule
// (including the overlapping "if" cases that only matter on meshes narrower
// than the stencil) is kept as in the scripts because it defines the format.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <sys/stat.h>

#include "internal.hpp"

namespace pda {

double round14(double v) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.14f", v);
  return std::strtod(buf, nullptr);
}

// hasBd{Left,Front,Right,Back}{1,2,3}d (mesh_ccu.hpp:161-296): a row is near
// the boundary if any stencil neighbour is outside the domain.
void Mesh::classify() {
  inner.clear();
  nearBd.clear();
  for (int64_t r = 0; r < sampleMeshSize; ++r) {
    bool bd = false;
    for (int c = 1; c < ncols; ++c)
      if (g(r, c) == -1) bd = true;
    if (bd)
      nearBd.push_back((int32_t)r);
    else
      inner.push_back((int32_t)r);
  }
  // checkIfFullyPeriodic (mesh_ccu.hpp:331-342)
  fullyPeriodic = true;
  for (int64_t r = 0; r < sampleMeshSize && fullyPeriodic; ++r)
    for (int c = 0; c < ncols; ++c)
      if (g(r, c) < 0) {
        fullyPeriodic = false;
        break;
      }
}

// ---------------------------------------------------------------- generators
namespace {

void graph1d(std::vector<int32_t> &G, int nx, int st, bool p) {
  const int nn = st - 1;
  G.assign((size_t)nx * (nn + 1), 0);
  for (int i = 0; i < nx; ++i) {
    int32_t t[6] = {0, 0, 0, 0, 0, 0};
    if (st == 3) {
      if (i == 0) t[0] = p ? i + nx - 1 : -1;
      if (i > 0) t[0] = i - 1;
      if (i == nx - 1) t[1] = p ? i - nx + 1 : -1;
      if (i < nx - 1) t[1] = i + 1;
    } else if (st == 5) {
      if (i == 0) { t[0] = p ? nx - 1 : -1; t[2] = p ? nx - 2 : -1; }
      else if (i == 1) { t[0] = 0; t[2] = p ? nx - 1 : -1; }
      else if (i > 1) { t[0] = i - 1; t[2] = i - 2; }
      if (i == nx - 1) { t[1] = p ? 0 : -1; t[3] = p ? 1 : -1; }
      if (i == nx - 2) { t[1] = nx - 1; t[3] = p ? 0 : -1; }
      if (i < nx - 2) { t[1] = i + 1; t[3] = i + 2; }
    } else {
      if (i == 0) { t[0] = p ? nx - 1 : -1; t[2] = p ? nx - 2 : -1; t[4] = p ? nx - 3 : -1; }
      else if (i == 1) { t[0] = 0; t[2] = p ? nx - 1 : -1; t[4] = p ? nx - 2 : -1; }
      else if (i == 2) { t[0] = i - 1; t[2] = i - 2; t[4] = p ? nx - 1 : -1; }
      else if (i > 2) { t[0] = i - 1; t[2] = i - 2; t[4] = i - 3; }
      if (i == nx - 1) { t[1] = p ? 0 : -1; t[3] = p ? 1 : -1; t[5] = p ? 2 : -1; }
      if (i == nx - 2) { t[1] = nx - 1; t[3] = p ? 0 : -1; t[5] = p ? 1 : -1; }
      if (i == nx - 3) { t[1] = nx - 2; t[3] = nx - 1; t[5] = p ? 0 : -1; }
      if (i < nx - 3) { t[1] = i + 1; t[3] = i + 2; t[5] = i + 3; }
    }
    G[(size_t)i * (nn + 1)] = i;
    for (int k = 0; k < nn; ++k) G[(size_t)i * (nn + 1) + 1 + k] = t[k];
  }
}

void graph2d(std::vector<int32_t> &G, int Nx, int Ny, int st, bool pX, bool pY) {
  const int nn = 2 * (st - 1);
  const int64_t N = (int64_t)Nx * Ny;
  G.assign((size_t)N * (nn + 1), 0);
  auto id = [&](int64_t gi, int64_t gj) { return (int32_t)(gj * Nx + gi); };
  for (int64_t iPt = 0; iPt < N; ++iPt) {
    const int64_t gi = iPt % Nx, gj = iPt / Nx;
    int32_t t[12] = {0};
    if (st == 3) {
      if (gi == 0) t[0] = pX ? (int32_t)(iPt + Nx - 1) : -1;
      if (gi > 0) t[0] = (int32_t)(iPt - 1);
      if (gj == Ny - 1) t[1] = pY ? (int32_t)(iPt - (int64_t)Nx * (Ny - 1)) : -1;
      if (gj < Ny - 1) t[1] = (int32_t)(iPt + Nx);
      if (gi == Nx - 1) t[2] = pX ? (int32_t)(iPt - Nx + 1) : -1;
      if (gi < Nx - 1) t[2] = (int32_t)(iPt + 1);
      if (gj == 0) t[3] = pY ? (int32_t)(iPt + (int64_t)Nx * (Ny - 1)) : -1;
      if (gj > 0) t[3] = (int32_t)(iPt - Nx);
    } else if (st == 5) {
      if (gi == 0) { t[0] = pX ? id(Nx - 1, gj) : -1; t[4] = pX ? id(Nx - 2, gj) : -1; }
      else if (gi == 1) { t[0] = id(0, gj); t[4] = pX ? id(Nx - 1, gj) : -1; }
      else if (gi > 1) { t[0] = id(gi - 1, gj); t[4] = id(gi - 2, gj); }
      if (gj == Ny - 1) { t[1] = pY ? id(gi, 0) : -1; t[5] = pY ? id(gi, 1) : -1; }
      if (gj == Ny - 2) { t[1] = id(gi, Ny - 1); t[5] = pY ? id(gi, 0) : -1; }
      if (gj < Ny - 2) { t[1] = id(gi, gj + 1); t[5] = id(gi, gj + 2); }
      if (gi == Nx - 1) { t[2] = pX ? id(0, gj) : -1; t[6] = pX ? id(1, gj) : -1; }
      if (gi == Nx - 2) { t[2] = id(Nx - 1, gj); t[6] = pX ? id(0, gj) : -1; }
      if (gi < Nx - 2) { t[2] = id(gi + 1, gj); t[6] = id(gi + 2, gj); }
      if (gj == 0) { t[3] = pY ? id(gi, Ny - 1) : -1; t[7] = pY ? id(gi, Ny - 2) : -1; }
      if (gj == 1) { t[3] = id(gi, 0); t[7] = pY ? id(gi, Ny - 1) : -1; }
      if (gj > 1) { t[3] = id(gi, gj - 1); t[7] = id(gi, gj - 2); }
    } else {
      if (gi == 0) { t[0] = pX ? id(Nx - 1, gj) : -1; t[4] = pX ? id(Nx - 2, gj) : -1; t[8] = pX ? id(Nx - 3, gj) : -1; }
      else if (gi == 1) { t[0] = id(0, gj); t[4] = pX ? id(Nx - 1, gj) : -1; t[8] = pX ? id(Nx - 2, gj) : -1; }
      else if (gi == 2) { t[0] = id(gi - 1, gj); t[4] = id(gi - 2, gj); t[8] = pX ? id(Nx - 1, gj) : -1; }
      else if (gi > 2) { t[0] = id(gi - 1, gj); t[4] = id(gi - 2, gj); t[8] = id(gi - 3, gj); }
      if (gj == Ny - 1) { t[1] = pY ? id(gi, 0) : -1; t[5] = pY ? id(gi, 1) : -1; t[9] = pY ? id(gi, 2) : -1; }
      if (gj == Ny - 2) { t[1] = id(gi, Ny - 1); t[5] = pY ? id(gi, 0) : -1; t[9] = pY ? id(gi, 1) : -1; }
      if (gj == Ny - 3) { t[1] = id(gi, Ny - 2); t[5] = id(gi, Ny - 1); t[9] = pY ? id(gi, 0) : -1; }
      if (gj < Ny - 3) { t[1] = id(gi, gj + 1); t[5] = id(gi, gj + 2); t[9] = id(gi, gj + 3); }
      if (gi == Nx - 1) { t[2] = pX ? id(0, gj) : -1; t[6] = pX ? id(1, gj) : -1; t[10] = pX ? id(2, gj) : -1; }
      if (gi == Nx - 2) { t[2] = id(Nx - 1, gj); t[6] = pX ? id(0, gj) : -1; t[10] = pX ? id(1, gj) : -1; }
      if (gi == Nx - 3) { t[2] = id(Nx - 2, gj); t[6] = id(Nx - 1, gj); t[10] = pX ? id(0, gj) : -1; }
      if (gi < Nx - 3) { t[2] = id(gi + 1, gj); t[6] = id(gi + 2, gj); t[10] = id(gi + 3, gj); }
      if (gj == 0) { t[3] = pY ? id(gi, Ny - 1) : -1; t[7] = pY ? id(gi, Ny - 2) : -1; t[11] = pY ? id(gi, Ny - 3) : -1; }
      if (gj == 1) { t[3] = id(gi, 0); t[7] = pY ? id(gi, Ny - 1) : -1; t[11] = pY ? id(gi, Ny - 2) : -1; }
      if (gj == 2) { t[3] = id(gi, 1); t[7] = id(gi, 0); t[11] = pY ? id(gi, Ny - 1) : -1; }
      if (gj > 2) { t[3] = id(gi, gj - 1); t[7] = id(gi, gj - 2); t[11] = id(gi, gj - 3); }
    }
    G[(size_t)iPt * (nn + 1)] = (int32_t)iPt;
    for (int k = 0; k < nn; ++k) G[(size_t)iPt * (nn + 1) + 1 + k] = t[k];
  }
}

// 3D: stencil 3 and 5 follow natural_order_mesh_3d.py; stencil 7 extends the
// same rule with a third layer in columns 13-18 = l2,f2,r2,ba2,bot2,top2.
void graph3d(std::vector<int32_t> &G, int Nx, int Ny, int Nz, int st, bool pX, bool pY, bool pZ) {
  const int nn = 3 * (st - 1);
  const int64_t N = (int64_t)Nx * Ny * Nz;
  G.assign((size_t)N * (nn + 1), 0);
  auto id = [&](int64_t gi, int64_t gj, int64_t gk) {
    return (int32_t)(gk * (int64_t)Nx * Ny + gj * Nx + gi);
  };
  for (int64_t iPt = 0; iPt < N; ++iPt) {
    const int64_t gi = iPt % ((int64_t)Nx * Ny) % Nx;
    const int64_t gj = (iPt % ((int64_t)Nx * Ny)) / Nx;
    const int64_t gk = iPt / ((int64_t)Nx * Ny);
    int32_t t[18] = {0};
    if (st == 3) {
      if (gi == 0) t[0] = pX ? id(Nx - 1, gj, gk) : -1;
      if (gi > 0) t[0] = id(gi - 1, gj, gk);
      if (gj == Ny - 1) t[1] = pY ? id(gi, 0, gk) : -1;
      if (gj < Ny - 1) t[1] = id(gi, gj + 1, gk);
      if (gi == Nx - 1) t[2] = pX ? id(0, gj, gk) : -1;
      if (gi < Nx - 1) t[2] = id(gi + 1, gj, gk);
      if (gj == 0) t[3] = pY ? id(gi, Ny - 1, gk) : -1;
      if (gj > 0) t[3] = id(gi, gj - 1, gk);
      if (gk == 0) t[4] = pZ ? id(gi, gj, Nz - 1) : -1;
      if (gk > 0) t[4] = id(gi, gj, gk - 1);
      if (gk == Nz - 1) t[5] = pZ ? id(gi, gj, 0) : -1;
      if (gk < Nz - 1) t[5] = id(gi, gj, gk + 1);
    } else {
      // layers L = 1 (st 5) or 2 (st 7); per-axis rule: for the "minus"
      // neighbour at distance d, d <= g uses the interior cell, otherwise
      // the periodic wrap or -1; same for the "plus" side.
      const int L = (st - 1) / 2;
      auto minus = [&](int64_t c, int d, int64_t n, bool p) -> int64_t {
        if (c - d >= 0) return c - d;
        return p ? c - d + n : -1;
      };
      auto plus = [&](int64_t c, int d, int64_t n, bool p) -> int64_t {
        if (c + d <= n - 1) return c + d;
        return p ? c + d - n : -1;
      };
      for (int d = 1; d <= L; ++d) {
        const int off = 6 * (d - 1);
        int64_t v;
        v = minus(gi, d, Nx, pX); t[off + 0] = v < 0 ? -1 : id(v, gj, gk);
        v = plus(gj, d, Ny, pY);  t[off + 1] = v < 0 ? -1 : id(gi, v, gk);
        v = plus(gi, d, Nx, pX);  t[off + 2] = v < 0 ? -1 : id(v, gj, gk);
        v = minus(gj, d, Ny, pY); t[off + 3] = v < 0 ? -1 : id(gi, v, gk);
        v = minus(gk, d, Nz, pZ); t[off + 4] = v < 0 ? -1 : id(gi, gj, v);
        v = plus(gk, d, Nz, pZ);  t[off + 5] = v < 0 ? -1 : id(gi, gj, v);
      }
    }
    G[(size_t)iPt * (nn + 1)] = (int32_t)iPt;
    for (int k = 0; k < nn; ++k) G[(size_t)iPt * (nn + 1) + 1 + k] = t[k];
  }
}

}  // namespace

Mesh mesh_generate_full(const int nIn[3], const double bd[6], int st, const int per[3]) {
  PDA_REQUIRE(st == 3 || st == 5 || st == 7, PDA_ERR_INVALID_ARGUMENT, "stencil size must be 3, 5 or 7");
  const int Nx = nIn[0], Ny = nIn[1] > 0 ? nIn[1] : 1, Nz = nIn[2] > 0 ? nIn[2] : 1;
  PDA_REQUIRE(Nx >= 1 && Ny >= 1 && Nz >= 1, PDA_ERR_INVALID_ARGUMENT, "cell counts must be positive");
  int dim;
  if (Ny == 1 && Nz == 1) dim = 1;
  else if (Nz == 1) dim = 2;
  else dim = 3;
  PDA_REQUIRE((int64_t)Nx * Ny * Nz < (int64_t)INT32_MAX / 8, PDA_ERR_INVALID_ARGUMENT,
              "mesh too large for int32 cell ids");
  Mesh m;
  m.dim = dim;
  m.stencil = st;
  m.n[0] = Nx;
  m.n[1] = Ny;
  m.n[2] = Nz;
  for (int a = 0; a < 3; ++a) m.periodic[a] = (a < dim) ? (per[a] ? 1 : 0) : 0;
  const int64_t N = (int64_t)Nx * Ny * Nz;
  m.stencilMeshSize = m.sampleMeshSize = N;
  m.ncols = 1 + (st - 1) * dim;
  // create_full_mesh.py:37-41: L = bounds, dx = L/N
  const double dxr = (bd[1] - bd[0]) / Nx;
  const double dyr = (bd[3] - bd[2]) / Ny;
  const double dzr = (bd[5] - bd[4]) / Nz;
  m.x.resize(N);
  m.y.resize(N);
  m.z.resize(N);
  if (dim == 1) {
    const double ox = bd[0] + 0.5 * dxr;
    for (int64_t i = 0; i < N; ++i) {
      m.x[i] = round14(ox + (double)i * dxr);
      m.y[i] = 0.0;
      m.z[i] = 0.0;
    }
    graph1d(m.graph, Nx, st, m.periodic[0]);
  } else if (dim == 2) {
    const double ox = bd[0] + 0.5 * dxr, oy = bd[2] + 0.5 * dyr;
    for (int64_t i = 0; i < N; ++i) {
      const int64_t gi = i % Nx, gj = i / Nx;
      m.x[i] = round14(ox + (double)gi * dxr);
      m.y[i] = round14(oy + (double)gj * dyr);
      m.z[i] = 0.0;
    }
    graph2d(m.graph, Nx, Ny, st, m.periodic[0], m.periodic[1]);
  } else {
    const double ox = bd[0] + 0.5 * dxr, oy = bd[2] + 0.5 * dyr, oz = bd[4] + 0.5 * dzr;
    for (int64_t i = 0; i < N; ++i) {
      const int64_t gi = i % ((int64_t)Nx * Ny) % Nx;
      const int64_t gj = (i % ((int64_t)Nx * Ny)) / Nx;
      const int64_t gk = i / ((int64_t)Nx * Ny);
      m.x[i] = round14(ox + (double)gi * dxr);
      m.y[i] = round14(oy + (double)gj * dyr);
      m.z[i] = round14(oz + (double)gk * dzr);
    }
    graph3d(m.graph, Nx, Ny, Nz, st, m.periodic[0], m.periodic[1], m.periodic[2]);
  }
  // read_mesh_info: dx parsed from "%.14f" text, dxInv = 1/dx
  const double d[3] = {dxr, dyr, dzr};
  for (int a = 0; a < 3; ++a) {
    if (a < dim) {
      m.dx[a] = round14(d[a]);
      m.dxInv[a] = 1.0 / m.dx[a];
    }
  }
  for (int k = 0; k < 6; ++k) m.bounds[k] = bd[k];
  m.hasBounds = true;
  m.structured = true;
  m.classify();
  return m;
}

// ------------------------------------------------------------------ files
namespace {
bool file_exists(const std::string &p) {
  struct stat sb;
  return ::stat(p.c_str(), &sb) == 0;
}
}  // namespace

Mesh mesh_load(const std::string &dir) {
  Mesh m;
  const std::string fi = dir + "/info.dat", fc = dir + "/connectivity.dat", fx = dir + "/coordinates.dat";
  PDA_REQUIRE(file_exists(fi), PDA_ERR_IO, "file not found " + fi);
  PDA_REQUIRE(file_exists(fc), PDA_ERR_IO, "file not found " + fc);
  PDA_REQUIRE(file_exists(fx), PDA_ERR_IO, "file not found " + fx);
  int nInfo[3] = {1, 1, 1};
  bool haveN = false;
  {
    std::ifstream src(fi);
    std::string line;
    bool bset[6] = {false, false, false, false, false, false};
    while (std::getline(src, line)) {
      std::istringstream ss(line);
      std::string key, val;
      ss >> key >> val;
      if (key.empty()) continue;
      try {
        if (key == "dim") m.dim = std::stoi(val);
        else if (key == "dx") { m.dx[0] = std::stod(val); m.dxInv[0] = 1.0 / m.dx[0]; }
        else if (key == "dy") { m.dx[1] = std::stod(val); m.dxInv[1] = 1.0 / m.dx[1]; }
        else if (key == "dz") { m.dx[2] = std::stod(val); m.dxInv[2] = 1.0 / m.dx[2]; }
        else if (key == "sampleMeshSize") m.sampleMeshSize = std::stoll(val);
        else if (key == "stencilMeshSize") m.stencilMeshSize = std::stoll(val);
        else if (key == "stencilSize") m.stencil = std::stoi(val);
        else if (key == "nx") { nInfo[0] = std::stoi(val); haveN = true; }
        else if (key == "ny") nInfo[1] = std::stoi(val);
        else if (key == "nz") nInfo[2] = std::stoi(val);
        else if (key == "xMin") { m.bounds[0] = std::stod(val); bset[0] = true; }
        else if (key == "xMax") { m.bounds[1] = std::stod(val); bset[1] = true; }
        else if (key == "yMin") { m.bounds[2] = std::stod(val); bset[2] = true; }
        else if (key == "yMax") { m.bounds[3] = std::stod(val); bset[3] = true; }
        else if (key == "zMin") { m.bounds[4] = std::stod(val); bset[4] = true; }
        else if (key == "zMax") { m.bounds[5] = std::stod(val); bset[5] = true; }
      } catch (const std::exception &) {
        throw Error(PDA_ERR_IO, "malformed entry in " + fi + ": " + line);
      }
    }
    m.hasBounds = bset[0] && bset[1];
  }
  PDA_REQUIRE(m.dim >= 1 && m.dim <= 3, PDA_ERR_IO, "info.dat: invalid dim");
  PDA_REQUIRE(m.stencil == 3 || m.stencil == 5 || m.stencil == 7, PDA_ERR_IO, "info.dat: invalid stencilSize");
  PDA_REQUIRE(m.sampleMeshSize > 0 && m.stencilMeshSize > 0, PDA_ERR_IO, "info.dat: invalid mesh sizes");
  m.ncols = 1 + (m.stencil - 1) * m.dim;
  m.graph.assign((size_t)m.sampleMeshSize * m.ncols, 0);
  {
    std::FILE *f = std::fopen(fc.c_str(), "r");
    PDA_REQUIRE(f, PDA_ERR_IO, "cannot open " + fc);
    const size_t total = m.graph.size();
    size_t k = 0;
    long v;
    while (k < total && std::fscanf(f, "%ld", &v) == 1) m.graph[k++] = (int32_t)v;
    std::fclose(f);
    PDA_REQUIRE(k == total, PDA_ERR_IO, "connectivity.dat: fewer entries than sampleMeshSize x columns");
  }
  for (int64_t r = 0; r < m.sampleMeshSize; ++r)
    for (int c = 0; c < m.ncols; ++c) {
      const int32_t v = m.g(r, c);
      PDA_REQUIRE(v >= -1 && v < m.stencilMeshSize && (c > 0 ? true : v >= 0), PDA_ERR_IO,
                  "connectivity.dat: cell id out of range");
    }
  m.x.assign(m.stencilMeshSize, 0.0);
  m.y.assign(m.stencilMeshSize, 0.0);
  m.z.assign(m.stencilMeshSize, 0.0);
  {
    std::ifstream src(fx);
    std::string line;
    while (std::getline(src, line)) {
      std::istringstream ss(line);
      std::string a, b, c, d;
      if (!(ss >> a)) continue;
      ss >> b >> c;
      long gid = std::stol(a);
      PDA_REQUIRE(gid >= 0 && gid < m.stencilMeshSize, PDA_ERR_IO, "coordinates.dat: gid out of range");
      m.x[gid] = std::stod(b);
      m.y[gid] = std::stod(c);
      if (m.dim == 3) {
        ss >> d;
        m.z[gid] = std::stod(d);
      }
    }
  }
  m.classify();
  mesh_detect_structure(m, nInfo, haveN);
  return m;
}

// A loaded mesh takes the structured fast path only if it is a full mesh
// whose graph equals the natural-order graph for its size and periodicity.
void mesh_detect_structure(Mesh &m, const int nInfo[3], bool haveN) {
  m.structured = false;
  if (!haveN || m.sampleMeshSize != m.stencilMeshSize) return;
  int n[3] = {nInfo[0], m.dim >= 2 ? nInfo[1] : 1, m.dim == 3 ? nInfo[2] : 1};
  if ((int64_t)n[0] * n[1] * n[2] != m.sampleMeshSize) return;
  // periodicity from the first cell's minus-neighbours
  int per[3] = {0, 0, 0};
  if (m.dim == 1) per[0] = m.g(0, 1) != -1;
  else if (m.dim == 2) { per[0] = m.g(0, 1) != -1; per[1] = m.g(0, 4) != -1; }
  else { per[0] = m.g(0, 1) != -1; per[1] = m.g(0, 4) != -1; per[2] = m.g(0, 5) != -1; }
  std::vector<int32_t> G;
  if (m.dim == 1) graph1d(G, n[0], m.stencil, per[0]);
  else if (m.dim == 2) graph2d(G, n[0], n[1], m.stencil, per[0], per[1]);
  else graph3d(G, n[0], n[1], n[2], m.stencil, per[0], per[1], per[2]);
  if (G != m.graph) return;
  for (int a = 0; a < 3; ++a) {
    m.n[a] = n[a];
    m.periodic[a] = per[a];
  }
  m.structured = true;
}

void mesh_write(const Mesh &m, const std::string &dir) {
  ::mkdir(dir.c_str(), 0755);
  {
    std::FILE *f = std::fopen((dir + "/info.dat").c_str(), "w");
    PDA_REQUIRE(f, PDA_ERR_IO, "cannot write " + dir + "/info.dat");
    const bool full = m.structured && m.sampleMeshSize == m.stencilMeshSize;
    std::fprintf(f, "dim %1d\n", m.dim);
    const char *nm[6] = {"xMin", "xMax", "yMin", "yMax", "zMin", "zMax"};
    for (int k = 0; k < 2 * m.dim; ++k) std::fprintf(f, "%s %.14f\n", nm[k], m.bounds[k]);
    const char *dn[3] = {"dx", "dy", "dz"};
    for (int a = 0; a < m.dim; ++a) std::fprintf(f, "%s %.14f\n", dn[a], m.dx[a]);
    std::fprintf(f, "sampleMeshSize %8lld\n", (long long)m.sampleMeshSize);
    std::fprintf(f, "stencilMeshSize %8lld\n", (long long)m.stencilMeshSize);
    std::fprintf(f, "stencilSize %2d\n", m.stencil);
    if (full) {
      const char *nn[3] = {"nx", "ny", "nz"};
      for (int a = 0; a < m.dim; ++a) std::fprintf(f, "%s %8d\n", nn[a], m.n[a]);
    }
    std::fclose(f);
  }
  {
    std::FILE *f = std::fopen((dir + "/connectivity.dat").c_str(), "w");
    PDA_REQUIRE(f, PDA_ERR_IO, "cannot write connectivity.dat");
    std::vector<char> buf;
    for (int64_t r = 0; r < m.sampleMeshSize; ++r) {
      for (int c = 0; c < m.ncols; ++c) std::fprintf(f, "%8d ", m.g(r, c));
      std::fputc('\n', f);
    }
    std::fclose(f);
  }
  {
    std::FILE *f = std::fopen((dir + "/coordinates.dat").c_str(), "w");
    PDA_REQUIRE(f, PDA_ERR_IO, "cannot write coordinates.dat");
    for (int64_t i = 0; i < m.stencilMeshSize; ++i) {
      std::fprintf(f, "%8lld ", (long long)i);
      std::fprintf(f, "%.14f ", m.x[i]);
      std::fprintf(f, "%.14f ", m.y[i]);
      if (m.dim == 3) std::fprintf(f, "%.14f ", m.z[i]);
      std::fputc('\n', f);
    }
    std::fclose(f);
  }
}

// ----------------------------------------------------------- binary files
// One little-endian file: a fixed header, the graph (int32, row-major), the
// x and y coordinates (and z in 3D) as doubles, then a 64-bit checksum of
// every byte before it.  The header carries what info.dat carries plus the
// structured-mesh descriptor, so loading needs no graph comparison.
namespace {
constexpr char kBinMagic[8] = {'P', 'D', 'A', 'M', 'E', 'S', 'H', '1'};
constexpr uint32_t kBinByteOrder = 0x01020304u;

struct BinHeader {
  char magic[8];
  uint32_t byteOrder;
  uint32_t headerBytes;
  int32_t dim, stencil, ncols, structured;
  int64_t stencilMeshSize, sampleMeshSize;
  double dx[3];
  double bounds[6];
  int32_t hasBounds, reserved;
  int32_t n[3], periodic[3];
};
static_assert(sizeof(BinHeader) % 8 == 0, "header keeps the arrays 8-byte aligned");

// 64-bit multiply-xorshift over 8-byte words (a tail shorter than 8 bytes is
// zero-padded): detects truncation and corruption, not tampering
struct Checksum {
  uint64_t h = 0x9E3779B97F4A7C15ull;
  void add(const void *data, size_t bytes) {
    const unsigned char *c = static_cast<const unsigned char *>(data);
    size_t k = 0;
    for (; k + 8 <= bytes; k += 8) {
      uint64_t w;
      std::memcpy(&w, c + k, 8);
      word(w);
    }
    if (k < bytes) {
      uint64_t w = 0;
      std::memcpy(&w, c + k, bytes - k);
      word(w);
    }
  }
  void word(uint64_t w) {
    h ^= w + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xFF51AFD7ED558CCDull;
    h ^= h >> 33;
  }
};

size_t graph_bytes(const Mesh &m) { return (size_t)m.sampleMeshSize * m.ncols * sizeof(int32_t); }
size_t pad8(size_t b) { return (b + 7) / 8 * 8; }
}  // namespace

void mesh_write_binary(const Mesh &m, const std::string &path) {
  BinHeader h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, kBinMagic, 8);
  h.byteOrder = kBinByteOrder;
  h.headerBytes = sizeof(BinHeader);
  h.dim = m.dim;
  h.stencil = m.stencil;
  h.ncols = m.ncols;
  h.structured = m.structured ? 1 : 0;
  h.stencilMeshSize = m.stencilMeshSize;
  h.sampleMeshSize = m.sampleMeshSize;
  for (int a = 0; a < 3; ++a) {
    h.dx[a] = m.dx[a];
    h.n[a] = m.n[a];
    h.periodic[a] = m.periodic[a];
  }
  for (int k = 0; k < 6; ++k) h.bounds[k] = m.bounds[k];
  h.hasBounds = m.hasBounds ? 1 : 0;
  std::FILE *f = std::fopen(path.c_str(), "wb");
  PDA_REQUIRE(f, PDA_ERR_IO, "cannot write " + path);
  Checksum cs;
  bool ok = true;
  auto put = [&](const void *p, size_t bytes) {
    if (bytes == 0 || !ok) return;
    ok = std::fwrite(p, 1, bytes, f) == bytes;
    cs.add(p, bytes);
  };
  put(&h, sizeof h);
  put(m.graph.data(), graph_bytes(m));
  const char zeros[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  put(zeros, pad8(graph_bytes(m)) - graph_bytes(m));
  const size_t nc = (size_t)m.stencilMeshSize * sizeof(double);
  put(m.x.data(), nc);
  put(m.y.data(), nc);
  if (m.dim == 3) put(m.z.data(), nc);
  const uint64_t sum = cs.h;
  if (ok) ok = std::fwrite(&sum, 1, 8, f) == 8;
  ok = (std::fclose(f) == 0) && ok;
  PDA_REQUIRE(ok, PDA_ERR_IO, "write failed: " + path);
}

Mesh mesh_load_binary(const std::string &path) {
  std::FILE *f = std::fopen(path.c_str(), "rb");
  PDA_REQUIRE(f, PDA_ERR_IO, "file not found " + path);
  struct Closer {
    std::FILE *f;
    ~Closer() { std::fclose(f); }
  } closer{f};
  std::fseek(f, 0, SEEK_END);
  const long long fileBytes = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  BinHeader h;
  PDA_REQUIRE(fileBytes >= (long long)sizeof h && std::fread(&h, 1, sizeof h, f) == sizeof h, PDA_ERR_IO,
              path + ": not a binary mesh file (too short)");
  PDA_REQUIRE(std::memcmp(h.magic, kBinMagic, 8) == 0, PDA_ERR_IO, path + ": not a binary mesh file");
  PDA_REQUIRE(h.byteOrder == kBinByteOrder, PDA_ERR_IO, path + ": written with another byte order");
  PDA_REQUIRE(h.headerBytes == sizeof h, PDA_ERR_IO, path + ": unsupported binary mesh version");
  PDA_REQUIRE(h.dim >= 1 && h.dim <= 3, PDA_ERR_IO, path + ": invalid dim");
  PDA_REQUIRE(h.stencil == 3 || h.stencil == 5 || h.stencil == 7, PDA_ERR_IO, path + ": invalid stencil size");
  PDA_REQUIRE(h.ncols == 1 + (h.stencil - 1) * h.dim, PDA_ERR_IO, path + ": invalid graph width");
  PDA_REQUIRE(h.sampleMeshSize > 0 && h.stencilMeshSize > 0 && h.sampleMeshSize <= h.stencilMeshSize &&
                  h.stencilMeshSize < (int64_t)1 << 31,
              PDA_ERR_IO, path + ": invalid mesh sizes");
  Mesh m;
  m.dim = h.dim;
  m.stencil = h.stencil;
  m.ncols = h.ncols;
  m.sampleMeshSize = h.sampleMeshSize;
  m.stencilMeshSize = h.stencilMeshSize;
  const size_t gb = graph_bytes(m), nc = (size_t)m.stencilMeshSize * sizeof(double);
  const size_t expect = sizeof h + pad8(gb) + nc * (m.dim == 3 ? 3 : 2) + 8;
  PDA_REQUIRE((size_t)fileBytes == expect, PDA_ERR_IO, path + ": truncated or oversized binary mesh file");
  Checksum cs;
  cs.add(&h, sizeof h);
  auto get = [&](void *p, size_t bytes) {
    if (bytes == 0) return;
    PDA_REQUIRE(std::fread(p, 1, bytes, f) == bytes, PDA_ERR_IO, path + ": read failed");
    cs.add(p, bytes);
  };
  m.graph.resize((size_t)m.sampleMeshSize * m.ncols);
  get(m.graph.data(), gb);
  char pad[8];
  get(pad, pad8(gb) - gb);
  m.x.resize(m.stencilMeshSize);
  m.y.resize(m.stencilMeshSize);
  m.z.assign(m.stencilMeshSize, 0.0);
  get(m.x.data(), nc);
  get(m.y.data(), nc);
  if (m.dim == 3) get(m.z.data(), nc);
  uint64_t sum = 0;
  PDA_REQUIRE(std::fread(&sum, 1, 8, f) == 8, PDA_ERR_IO, path + ": read failed");
  PDA_REQUIRE(sum == cs.h, PDA_ERR_IO, path + ": checksum mismatch (corrupt binary mesh file)");
  for (int64_t r = 0; r < m.sampleMeshSize; ++r)
    for (int c = 0; c < m.ncols; ++c) {
      const int32_t v = m.g(r, c);
      PDA_REQUIRE(v >= -1 && v < m.stencilMeshSize && (c > 0 ? true : v >= 0), PDA_ERR_IO,
                  path + ": cell id out of range");
    }
  for (int a = 0; a < 3; ++a) {
    m.dx[a] = h.dx[a];
    m.dxInv[a] = a < m.dim ? 1.0 / h.dx[a] : 0.0;
    m.n[a] = h.n[a];
    m.periodic[a] = h.periodic[a];
  }
  for (int k = 0; k < 6; ++k) m.bounds[k] = h.bounds[k];
  m.hasBounds = h.hasBounds != 0;
  m.classify();
  m.structured = h.structured != 0;
  if (m.structured)
    PDA_REQUIRE(m.sampleMeshSize == m.stencilMeshSize && (int64_t)m.n[0] * m.n[1] * m.n[2] == m.sampleMeshSize,
                PDA_ERR_IO, path + ": inconsistent structured-mesh descriptor");
  return m;
}

// create_sample_mesh.py:54-137
Mesh mesh_sample(const Mesh &full, const std::vector<int64_t> &gidsIn, std::vector<int64_t> *stencilOut) {
  PDA_REQUIRE(full.sampleMeshSize == full.stencilMeshSize, PDA_ERR_INVALID_ARGUMENT,
              "sample meshes are built from a full mesh");
  std::vector<int64_t> gids(gidsIn);
  std::sort(gids.begin(), gids.end());
  gids.erase(std::unique(gids.begin(), gids.end()), gids.end());
  for (int64_t g : gids)
    PDA_REQUIRE(g >= 0 && g < full.sampleMeshSize, PDA_ERR_INVALID_ARGUMENT, "sample gid out of range");
  std::vector<int64_t> st;
  for (int64_t g : gids) {
    st.push_back(g);
    for (int c = 1; c < full.ncols; ++c) {
      const int32_t j = full.g(g, c);
      if (j != -1) st.push_back(j);
    }
  }
  std::sort(st.begin(), st.end());
  st.erase(std::unique(st.begin(), st.end()), st.end());
  std::map<int64_t, int32_t> fm2sm;
  for (size_t i = 0; i < st.size(); ++i) fm2sm[st[i]] = (int32_t)i;
  Mesh m;
  m.dim = full.dim;
  m.stencil = full.stencil;
  m.ncols = full.ncols;
  for (int a = 0; a < 3; ++a) {
    m.dx[a] = full.dx[a];
    m.dxInv[a] = full.dxInv[a];
  }
  for (int k = 0; k < 6; ++k) m.bounds[k] = full.bounds[k];
  m.hasBounds = full.hasBounds;
  m.sampleMeshSize = (int64_t)gids.size();
  m.stencilMeshSize = (int64_t)st.size();
  m.graph.assign((size_t)m.sampleMeshSize * m.ncols, 0);
  for (size_t r = 0; r < gids.size(); ++r) {
    m.graph[r * m.ncols] = fm2sm[gids[r]];
    for (int c = 1; c < m.ncols; ++c) {
      const int32_t j = full.g(gids[r], c);
      m.graph[r * m.ncols + c] = (j == -1) ? -1 : fm2sm[j];
    }
  }
  // rows are written sorted by their stencil-mesh id, which is monotone in
  // the sorted sample gids, so the row order above already matches.
  m.x.resize(st.size());
  m.y.resize(st.size());
  m.z.resize(st.size());
  for (size_t i = 0; i < st.size(); ++i) {
    m.x[i] = full.x[st[i]];
    m.y[i] = full.y[st[i]];
    m.z[i] = full.z[st[i]];
  }
  m.classify();
  m.structured = false;
  if (stencilOut) *stencilOut = st;
  return m;
}

}  // namespace pda
