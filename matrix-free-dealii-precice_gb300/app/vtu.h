// Solution output of the executables: the reference's output_results
// (include/solid_mechanics/mf_elasticity.h:2074-2126,
// include/heat_transfer/heat_transfer.h:854-880) writes solution_NNN.vtu with
// deal.II's DataOut: one higher-order Lagrange cell of degree p per mesh cell
// (write_higher_order_cells, build_patches with p subdivisions), the field
// evaluated at equispaced points of every cell, the solid on the displaced
// (Eulerian) geometry.  This writes the same content as a VTK XML
// UnstructuredGrid with raw appended data: VTK_LAGRANGE_HEXAHEDRON (72) or
// VTK_LAGRANGE_QUADRILATERAL (70) cells in VTK's point order, float64
// points and point data, float32 cell data.
#pragma once

#include <sys/stat.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mfgpu.h"

namespace mfapp
{
  // Gauss-Lobatto support points of FE_Q(p) on [0,1]
  inline std::vector<double>
  lobatto(int p)
  {
    std::vector<double> x(p + 1);
    x[0] = 0;
    x[p] = 1;
    for (int i = 1; i < p; ++i)
      {
        long double z = -std::cos(3.14159265358979323846L * i / p);
        for (int it = 0; it < 100; ++it)
          {
            long double p0 = 1, p1 = z;
            for (int k = 2; k <= p; ++k)
              {
                long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0             = p1;
                p1             = p2;
              }
            const long double dp = p * (z * p1 - p0) / (z * z - 1);
            const long double d2 = (2 * z * dp - p * (p + 1) * p1) / (1 - z * z);
            z -= dp / d2;
          }
        x[i] = double((1 + z) / 2);
      }
    return x;
  }

  // index of point (i,j,k) of an order-p Lagrange hexahedron in VTK's point
  // order: 8 vertices, 12 edges, 6 faces, then the interior (the order of
  // the VTK file format's higher-order cells)
  inline int
  vtk_hex_index(int i, int j, int k, int p)
  {
    const bool ib = i == 0 || i == p, jb = j == 0 || j == p, kb = k == 0 || k == p;
    const int  nb = int(ib) + int(jb) + int(kb);
    if (nb == 3)
      return (i ? (j ? 2 : 1) : (j ? 3 : 0)) + (k ? 4 : 0);
    int off = 8;
    const int e = p - 1; // interior points per edge
    if (nb == 2)
      {
        if (!ib) // edge along x
          return (i - 1) + (j ? 2 * e : 0) + (k ? 4 * e : 0) + off;
        if (!jb) // edge along y
          return (j - 1) + (i ? e : 3 * e) + (k ? 4 * e : 0) + off;
        off += 8 * e; // edge along z
        return (k - 1) + e * (i ? (j ? 3 : 1) : (j ? 2 : 0)) + off;
      }
    off += 12 * e;
    if (nb == 1)
      {
        if (ib) // x-normal face
          return (j - 1) + e * (k - 1) + (i ? e * e : 0) + off;
        off += 2 * e * e;
        if (jb) // y-normal face
          return (i - 1) + e * (k - 1) + (j ? e * e : 0) + off;
        off += 2 * e * e; // z-normal face
        return (i - 1) + e * (j - 1) + (k ? e * e : 0) + off;
      }
    off += 6 * e * e;
    return off + (i - 1) + e * ((j - 1) + e * (k - 1));
  }

  // the same for an order-p Lagrange quadrilateral
  inline int
  vtk_quad_index(int i, int j, int p)
  {
    const bool ib = i == 0 || i == p, jb = j == 0 || j == p;
    if (ib && jb)
      return i ? (j ? 2 : 1) : (j ? 3 : 0);
    const int e = p - 1;
    if (jb) // edge along x
      return 4 + (i - 1) + (j ? 2 * e : 0);
    if (ib) // edge along y
      return 4 + (j - 1) + (i ? e : 3 * e);
    return 4 + 4 * e + (i - 1) + e * (j - 1);
  }

  // file = solution_NNN.vtu; u: nodal values of nc components, component
  // blocked on the box's lexicographic node grid; displace: points at
  // x + u (the first dim components); cell_fields: constant cell data
  inline void
  write_vtu(const std::string &file, const mfgpu_mesh &m, int dim, int nc, const std::vector<double> &u,
            const std::string &name, bool displace, const std::vector<std::pair<std::string, double>> &cell_fields)
  {
    const int p = m.degree, n1 = p + 1;
    int       C[3] = {1, 1, 1}, Nn[3] = {1, 1, 1};
    double    h[3] = {1, 1, 1};
    for (int d = 0; d < dim; ++d)
      {
        C[d]  = m.repetitions[d] << m.n_refinements;
        Nn[d] = C[d] * p + 1;
        h[d]  = (m.upper[d] - m.lower[d]) / C[d];
      }
    const size_t n_nodes = size_t(Nn[0]) * Nn[1] * Nn[2];
    if (u.size() != n_nodes * size_t(nc))
      throw std::runtime_error("write_vtu: vector size does not match the mesh");
    const int    ppc     = dim == 3 ? n1 * n1 * n1 : n1 * n1; // points per cell
    const size_t n_cells = size_t(C[0]) * C[1] * C[2];
    const size_t n_pts   = n_cells * size_t(ppc);
    // E[a][i] = l_i(a/p): the GLL Lagrange basis at the equispaced points
    const std::vector<double> gl = lobatto(p);
    std::vector<double>       E(size_t(n1) * n1);
    for (int a = 0; a < n1; ++a)
      for (int i = 0; i < n1; ++i)
        {
          double l = 1, x = double(a) / p;
          for (int j = 0; j < n1; ++j)
            if (j != i)
              l *= (x - gl[j]) / (gl[i] - gl[j]);
          E[size_t(a) * n1 + i] = l;
        }
    const int            ncv = nc == 1 ? 1 : 3; // vectors are written with 3 components
    std::vector<double>  pts(n_pts * 3), val(n_pts * size_t(ncv), 0.0);
    std::vector<int64_t> conn(n_pts), offs(n_cells);
    std::vector<uint8_t> types(n_cells, uint8_t(dim == 3 ? 72 : 70));
    const int            nk = dim == 3 ? n1 : 1;
    std::vector<double>  t0(ppc), t1(ppc);
    std::vector<double>  cellv(size_t(nc) * ppc);
    for (int cz = 0; cz < C[2]; ++cz)
      for (int cy = 0; cy < C[1]; ++cy)
        for (int cx = 0; cx < C[0]; ++cx)
          {
            const size_t cell = size_t(cx) + size_t(C[0]) * (size_t(cy) + size_t(C[1]) * cz);
            const size_t base = cell * size_t(ppc);
            for (int c = 0; c < nc; ++c)
              {
                // nodal values of the cell, then E along x, y (and z)
                for (int k = 0; k < nk; ++k)
                  for (int j = 0; j < n1; ++j)
                    for (int i = 0; i < n1; ++i)
                      t0[size_t(i) + n1 * (j + size_t(n1) * k)] =
                        u[size_t(c) * n_nodes + size_t(cx * p + i) +
                          size_t(Nn[0]) * (size_t(cy * p + j) + size_t(Nn[1]) * size_t(dim == 3 ? cz * p + k : 0))];
                for (int dir = 0; dir < dim; ++dir)
                  {
                    const int st = dir == 0 ? 1 : (dir == 1 ? n1 : n1 * n1);
                    for (int q = 0; q < ppc; ++q)
                      {
                        const int a  = (q / st) % n1;
                        double    s  = 0;
                        const int b0 = q - a * st;
                        for (int i = 0; i < n1; ++i)
                          s += E[size_t(a) * n1 + i] * t0[size_t(b0 + i * st)];
                        t1[size_t(q)] = s;
                      }
                    t0.swap(t1);
                  }
                for (int q = 0; q < ppc; ++q)
                  cellv[size_t(c) * ppc + q] = t0[size_t(q)];
              }
            for (int k = 0; k < nk; ++k)
              for (int j = 0; j < n1; ++j)
                for (int i = 0; i < n1; ++i)
                  {
                    const int    q  = i + n1 * (j + n1 * k);
                    const size_t pt = base + size_t(dim == 3 ? vtk_hex_index(i, j, k, p) : vtk_quad_index(i, j, p));
                    const double x[3] = {m.lower[0] + (cx + double(i) / p) * h[0],
                                         m.lower[1] + (cy + double(j) / p) * h[1],
                                         dim == 3 ? m.lower[2] + (cz + double(k) / p) * h[2] : 0.0};
                    for (int d = 0; d < 3; ++d)
                      pts[pt * 3 + d] = x[d] + (displace && d < dim && d < nc ? cellv[size_t(d) * ppc + q] : 0.0);
                    for (int c = 0; c < nc; ++c)
                      val[pt * size_t(ncv) + c] = cellv[size_t(c) * ppc + q];
                  }
            for (int q = 0; q < ppc; ++q)
              conn[base + q] = int64_t(base + q);
            offs[cell] = int64_t(base + ppc);
          }

    // XML header with appended-data offsets, then the raw blocks (each a
    // UInt64 byte count and the bytes)
    struct Block
    {
      const void *ptr;
      uint64_t    bytes;
    };
    std::vector<Block>  blocks;
    std::vector<size_t> offsets;
    size_t              off = 0;
    auto                add = [&](const void *ptr, uint64_t bytes) {
      offsets.push_back(off);
      blocks.push_back({ptr, bytes});
      off += sizeof(uint64_t) + bytes;
      return offsets.back();
    };
    std::vector<std::vector<float>> cf(cell_fields.size(), std::vector<float>(n_cells));
    for (size_t f = 0; f < cell_fields.size(); ++f)
      for (auto &x : cf[f])
        x = float(cell_fields[f].second);
    std::string xml = "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" "
                      "byte_order=\"LittleEndian\" header_type=\"UInt64\">\n<UnstructuredGrid>\n";
    xml += "<Piece NumberOfPoints=\"" + std::to_string(n_pts) + "\" NumberOfCells=\"" + std::to_string(n_cells) +
           "\">\n";
    xml += std::string("<PointData ") + (ncv == 1 ? "Scalars" : "Vectors") + "=\"" + name + "\">\n";
    xml += "<DataArray type=\"Float64\" Name=\"" + name + "\" NumberOfComponents=\"" + std::to_string(ncv) +
           "\" format=\"appended\" offset=\"" + std::to_string(add(val.data(), val.size() * 8)) + "\"/>\n";
    xml += "</PointData>\n<CellData>\n";
    for (size_t f = 0; f < cell_fields.size(); ++f)
      xml += "<DataArray type=\"Float32\" Name=\"" + cell_fields[f].first + "\" format=\"appended\" offset=\"" +
             std::to_string(add(cf[f].data(), cf[f].size() * 4)) + "\"/>\n";
    xml += "</CellData>\n<Points>\n<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"appended\" "
           "offset=\"" +
           std::to_string(add(pts.data(), pts.size() * 8)) + "\"/>\n</Points>\n<Cells>\n";
    xml += "<DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\"" +
           std::to_string(add(conn.data(), conn.size() * 8)) + "\"/>\n";
    xml += "<DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"" +
           std::to_string(add(offs.data(), offs.size() * 8)) + "\"/>\n";
    xml += "<DataArray type=\"UInt8\" Name=\"types\" format=\"appended\" offset=\"" +
           std::to_string(add(types.data(), types.size())) + "\"/>\n";
    xml += "</Cells>\n</Piece>\n</UnstructuredGrid>\n<AppendedData encoding=\"raw\">\n_";
    std::FILE *fp = std::fopen(file.c_str(), "wb");
    if (!fp)
      throw std::runtime_error("can't create: " + file);
    std::fwrite(xml.data(), 1, xml.size(), fp);
    for (const Block &b : blocks)
      {
        std::fwrite(&b.bytes, sizeof(uint64_t), 1, fp);
        std::fwrite(b.ptr, 1, b.bytes, fp);
      }
    const char tail[] = "\n</AppendedData>\n</VTKFile>\n";
    std::fwrite(tail, 1, sizeof(tail) - 1, fp);
    std::fclose(fp);
  }

  // mkdir -p
  inline void
  make_dirs(const std::string &path)
  {
    std::string acc;
    for (size_t i = 0; i < path.size(); ++i)
      {
        acc += path[i];
        if (path[i] == '/' && acc.size() > 1)
          mkdir(acc.c_str(), 0755);
      }
    if (!acc.empty())
      mkdir(acc.c_str(), 0755);
  }

  // solution_NNN.vtu under an output folder ("" or ending in '/')
  inline std::string
  vtu_name(const std::string &folder, int number)
  {
    char buf[32];
    std::snprintf(buf, sizeof(buf), "solution_%03d.vtu", number);
    return folder + buf;
  }
} // namespace mfapp
