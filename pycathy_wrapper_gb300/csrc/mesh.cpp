// Host mesh construction; see mesh.h.
#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace cathy {

// ---------------------------------------------------------------------------
// DEM -> surface triangulation (triangoli.f semantics with DOSTEP = 1):
// nodes at the corners of active cells numbered row-major from the north-west
// corner, two triangles per active cell, node elevation = mean elevation of
// the incident triangles (tpnodi2d.f).
// ---------------------------------------------------------------------------
static bool surface_mesh(const cathy_dem_t& d, HostMesh& m,
                         std::vector<double>& zsurf) {
  const int nr = d.nrow, nc = d.ncol;
  std::vector<int32_t> corner((size_t)(nr + 1) * (nc + 1), 0);
  auto C = [&](int i, int j) -> int32_t& { return corner[(size_t)i * (nc + 1) + j]; };
  auto active = [&](int i, int j) { return d.dem[(size_t)i * nc + j] != 0.0; };
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nc; ++j)
      if (active(i, j)) C(i, j) = C(i + 1, j) = C(i + 1, j + 1) = C(i, j + 1) = 1;
  int id = 0;
  m.x.clear(); m.y.clear();
  for (int i = 0; i <= nr; ++i)
    for (int j = 0; j <= nc; ++j)
      if (C(i, j)) {
        C(i, j) = ++id;
        m.x.push_back(d.west + j * d.delta_x);
        m.y.push_back(d.south + (nr - i) * d.delta_y);
      }
  m.nnod = id;
  m.triang.clear();
  std::vector<double> elev;
  int zmax = 1;
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nc; ++j) {
      if (!active(i, j)) continue;
      const double e = d.dem[(size_t)i * nc + j] * d.factor;
      const int zn = d.zone ? d.zone[(size_t)i * nc + j] : 1;
      zmax = std::max(zmax, zn);
      const int a = C(i, j), b = C(i + 1, j), c = C(i + 1, j + 1), dd = C(i, j + 1);
      const int t1[3] = {a, b, c}, t2[3] = {a, c, dd};
      for (const int* t : {t1, t2}) {
        int s[3] = {t[0], t[1], t[2]};
        std::sort(s, s + 3);  // RIORD on triangles (grdsys.f)
        m.triang.insert(m.triang.end(), {s[0], s[1], s[2], zn});
        elev.push_back(e);
      }
    }
  m.ntri = (int)elev.size();
  m.nzone = zmax;
  // node elevation: unweighted mean over incident triangles
  zsurf.assign(m.nnod, 0.0);
  std::vector<int> cnt(m.nnod, 0);
  // accumulation order follows triangle order (as TPNODI2D)
  // note: TPNODI2D runs before RIORD, summation order over triangles is the
  // same either way.
  for (int t = 0; t < m.ntri; ++t)
    for (int q = 0; q < 3; ++q) {
      const int nd = m.triang[4 * t + q] - 1;
      zsurf[nd] += elev[t];
      cnt[nd] += 1;
    }
  for (int k = 0; k < m.nnod; ++k) {
    if (cnt[k] == 0) return false;
    zsurf[k] /= cnt[k];
  }
  // node areas: one third of each incident triangle's area (area2d.f)
  m.arenod.assign(m.nnod, 0.0);
  for (int t = 0; t < m.ntri; ++t) {
    const int* tr = &m.triang[4 * t];
    const double x1 = m.x[tr[0] - 1], y1 = m.y[tr[0] - 1], x2 = m.x[tr[1] - 1],
                 y2 = m.y[tr[1] - 1], x3 = m.x[tr[2] - 1], y3 = m.y[tr[2] - 1];
    // shoelace in the reference's summation order (areas.f)
    const double a3 = x1 * y2 + (x2 * y3 + (x3 * y1));
    const double a2 = x1 * y3 + (x2 * y1 + (x3 * y2));
    const double are = 0.5 * (((x1 * y2 + 0.0) + x2 * y3) + x3 * y1 -
                               (((x1 * y3 + 0.0) + x2 * y1) + x3 * y2));
    (void)a3; (void)a2;
    if (are == 0.0) return false;
    const double are3 = std::fabs(are) * (1.0 / 3.0);
    for (int q = 0; q < 3; ++q) m.arenod[tr[q] - 1] += are3;
  }
  return true;
}

bool node_map_types(const cathy_dem_t& d, const double* map, const HostMesh& m,
                    std::vector<int32_t>& out) {
  out.assign(m.nnod, 1);
  if (!map) return true;
  std::vector<double> sum(m.nnod, 0.0);
  std::vector<int> cnt(m.nnod, 0);
  // triangles come two per active cell in row-major cell order (build_mesh)
  int t = 0;
  for (int i = 0; i < d.nrow; ++i)
    for (int j = 0; j < d.ncol; ++j) {
      const size_t c = (size_t)i * d.ncol + j;
      if (d.dem[c] == 0.0) continue;
      if (map[c] == 0.0) return false;
      const double e = map[c] * d.factor;
      for (int h = 0; h < 2; ++h, ++t)
        for (int q = 0; q < 3; ++q) {
          const int nd = m.triang[4 * t + q] - 1;
          sum[nd] += e;
          cnt[nd] += 1;
        }
    }
  for (int k = 0; k < m.nnod; ++k) out[k] = (int32_t)(sum[k] / cnt[k]);
  return true;
}

bool build_mesh(const cathy_dem_t& d, int iopt, HostMesh& m) {
  // GEN3D's IVERT 3 takes a per-node depth map (gen3d.f:67-68), which the
  // DEM inputs here do not carry: refused, as are values GEN3D does not know
  if (d.ivert != 0 && d.ivert != 1 && d.ivert != 2 && d.ivert != 4) return false;
  m.nrow = d.nrow; m.ncol = d.ncol; m.nstr = d.nstr; m.iopt = iopt;
  std::vector<double> zs;
  if (!surface_mesh(d, m, zs)) return false;
  const int nnod = m.nnod, ntri = m.ntri, nstr = m.nstr;
  m.n = nnod * (nstr + 1);
  m.nt = 3 * ntri * nstr;
  const int n = m.n, nt = m.nt;
  // vertical extrusion: 3 tetrahedra per prism (gen3d.f:28-47)
  m.tetra.assign((size_t)5 * nt, 0);
  m.tet_layer.assign(nt, 0);
  for (int j = 1; j <= nstr; ++j)
    for (int i = 0; i < ntri; ++i) {
      const int* tr = &m.triang[4 * i];
      const size_t e = (size_t)3 * ((j - 1) * ntri + i);
      int32_t* t1 = &m.tetra[5 * e];
      int32_t* t2 = t1 + 5;
      int32_t* t3 = t1 + 10;
      const int lo = (j - 1) * nnod, hi = j * nnod;
      t1[0] = lo + tr[0]; t1[1] = lo + tr[1]; t1[2] = lo + tr[2]; t1[3] = hi + tr[0];
      t2[0] = hi + tr[0]; t2[1] = hi + tr[1]; t2[2] = hi + tr[2]; t2[3] = lo + tr[2];
      t3[0] = lo + tr[1]; t3[1] = lo + tr[2]; t3[2] = hi + tr[1]; t3[3] = hi + tr[0];
      t1[4] = t2[4] = t3[4] = tr[3];
      m.tet_layer[e] = m.tet_layer[e + 1] = m.tet_layer[e + 2] = j;
    }
  // layer elevations (gen3d.f:48-77)
  m.x.resize(n); m.y.resize(n); m.z.assign(n, 0.0);
  double zmin = 1.7e100;
  for (int i = 0; i < nnod; ++i) zmin = std::min(zmin, zs[i]);
  for (int i = 0; i < nnod; ++i) {
    m.z[i] = zs[i];
    const double zthick = (zs[i] - zmin) + d.base;
    double zr = 0.0;
    for (int j = 1; j <= nstr; ++j) {
      const int kk = j * nnod + i;
      m.x[kk] = m.x[i];
      m.y[kk] = m.y[i];
      zr = zr + d.zratio[j - 1];
      double zz;
      switch (d.ivert) {
        case 1: zz = zs[i] - zr * zthick; break;
        case 2: zz = zmin - zr * d.base; break;
        case 4: zz = (j == nstr) ? zmin - d.base : zs[i] - zr * d.base; break;
        default: zz = zs[i] - zr * d.base; break;  // IVERT 0
      }
      m.z[kk] = zz;
    }
  }
  // ascending node order inside each element for the symmetric scheme
  if (iopt == 1)
    for (int e = 0; e < nt; ++e) std::sort(&m.tetra[5 * e], &m.tetra[5 * e] + 4);
  // node -> element incidence (counting sort by node)
  m.inc_ptr.assign(n + 1, 0);
  for (int e = 0; e < nt; ++e)
    for (int k = 0; k < 4; ++k) m.inc_ptr[m.tetra[5 * e + k]]++;  // 1-based -> shift
  for (int i = 0; i < n; ++i) m.inc_ptr[i + 1] += m.inc_ptr[i];
  m.inc.assign(m.inc_ptr[n], 0);
  {
    std::vector<int32_t> fill(m.inc_ptr.begin(), m.inc_ptr.end() - 1);
    for (int e = 0; e < nt; ++e)
      for (int k = 0; k < 4; ++k) {
        const int nd = m.tetra[5 * e + k] - 1;
        m.inc[fill[nd]++] = e * 4 + k;
      }
  }
  for (int i = 0; i < n; ++i)
    if (m.inc_ptr[i + 1] == m.inc_ptr[i]) return false;
  // full CSR: union of the element node sets of each row, sorted
  m.rowptr.assign(n + 1, 0);
  m.cols.clear();
  m.cols.reserve((size_t)n * 16);
  std::vector<int32_t> buf;
  for (int i = 0; i < n; ++i) {
    buf.clear();
    for (int p = m.inc_ptr[i]; p < m.inc_ptr[i + 1]; ++p) {
      const int e = m.inc[p] >> 2;
      for (int k = 0; k < 4; ++k) buf.push_back(m.tetra[5 * e + k] - 1);
    }
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    m.cols.insert(m.cols.end(), buf.begin(), buf.end());
    m.rowptr[i + 1] = (int32_t)m.cols.size();
  }
  m.diag.assign(n, -1);
  m.down.assign(n, -1);
  m.up.assign(n, -1);
  for (int i = 0; i < n; ++i)
    for (int s = m.rowptr[i]; s < m.rowptr[i + 1]; ++s) {
      if (m.cols[s] == i) m.diag[i] = s;
      if (m.cols[s] == i + nnod) m.down[i] = s;
      if (m.cols[s] == i - nnod) m.up[i] = s;
    }
  level_schedule(n, m.rowptr, m.cols, true, m.lev_f_ptr, m.lev_f_rows);
  level_schedule(n, m.rowptr, m.cols, false, m.lev_b_ptr, m.lev_b_rows);
  return true;
}

void level_schedule(int n, const std::vector<int32_t>& rowptr,
                    const std::vector<int32_t>& cols, bool lower,
                    std::vector<int32_t>& lev_ptr, std::vector<int32_t>& rows) {
  std::vector<int32_t> lev(n, 0);
  int maxl = 0;
  if (lower) {
    for (int i = 0; i < n; ++i) {
      int l = 0;
      for (int s = rowptr[i]; s < rowptr[i + 1]; ++s)
        if (cols[s] < i) l = std::max(l, lev[cols[s]] + 1);
      lev[i] = l;
      maxl = std::max(maxl, l);
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int l = 0;
      for (int s = rowptr[i]; s < rowptr[i + 1]; ++s)
        if (cols[s] > i) l = std::max(l, lev[cols[s]] + 1);
      lev[i] = l;
      maxl = std::max(maxl, l);
    }
  }
  lev_ptr.assign(maxl + 2, 0);
  for (int i = 0; i < n; ++i) lev_ptr[lev[i] + 1]++;
  for (int l = 0; l <= maxl; ++l) lev_ptr[l + 1] += lev_ptr[l];
  rows.assign(n, 0);
  std::vector<int32_t> fill(lev_ptr.begin(), lev_ptr.end() - 1);
  for (int i = 0; i < n; ++i) rows[fill[lev[i]]++] = i;
}

void upper_to_full(int n, const int32_t* topol, const int32_t* ja,
                   std::vector<int32_t>& rowptr, std::vector<int32_t>& cols,
                   std::vector<int32_t>& up_slot_of_full) {
  // count: each stored (i,j) with j>i appears in rows i and j
  std::vector<int32_t> cnt(n + 1, 0);
  for (int i = 0; i < n; ++i)
    for (int s = topol[i] - 1; s < topol[i + 1] - 1; ++s) {
      const int j = ja[s] - 1;
      cnt[i]++;
      if (j != i) cnt[j]++;
    }
  rowptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) rowptr[i + 1] = rowptr[i] + cnt[i];
  cols.assign(rowptr[n], 0);
  up_slot_of_full.assign(rowptr[n], 0);
  std::vector<int32_t> fill(rowptr.begin(), rowptr.end() - 1);
  // rows are filled in increasing column order: lower entries come from
  // earlier rows' upper storage (visited in increasing row order), then the
  // row's own upper storage (diagonal first, increasing columns)
  for (int i = 0; i < n; ++i) {
    for (int s = topol[i] - 1; s < topol[i + 1] - 1; ++s) {
      const int j = ja[s] - 1;
      if (j == i) continue;
      cols[fill[j]] = i;
      up_slot_of_full[fill[j]] = s;
      fill[j]++;
    }
    for (int s = topol[i] - 1; s < topol[i + 1] - 1; ++s) {
      cols[fill[i]] = ja[s] - 1;
      up_slot_of_full[fill[i]] = s;
      fill[i]++;
    }
  }
}

}  // namespace cathy
