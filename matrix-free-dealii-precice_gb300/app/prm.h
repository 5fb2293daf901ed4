// Parameter files in deal.II ParameterHandler syntax ("subsection X",
// "set key = value", "end", '#' comments), restating the entries the
// reference declares (include/parameter/parameter_handling.h:16-331,
// include/parameter/precice_parameter.h:18-87).  Unknown subsections or
// entries are errors, as in ParameterHandler::parse_input; the preCICE
// section is parsed and ignored (the coupling is replaced by constant
// boundary data).
#pragma once

#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace mfapp
{
  inline std::string
  trim(const std::string &s)
  {
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos)
      return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
  }

  struct Prm
  {
    // "Section/Key" -> value
    std::map<std::string, std::string> values;

    // declared entries: section -> keys (with defaults)
    std::map<std::string, std::map<std::string, std::string>> declared;

    void
    declare(const std::string &section, const std::string &key, const std::string &def)
    {
      declared[section][key] = def;
    }

    void
    parse(const std::string &file)
    {
      std::ifstream in(file);
      if (!in)
        throw std::runtime_error("cannot open parameter file '" + file + "'");
      std::vector<std::string> stack;
      std::string              line;
      int                      lineno = 0;
      while (std::getline(in, line))
        {
          ++lineno;
          const size_t h = line.find('#');
          if (h != std::string::npos)
            line = line.substr(0, h);
          line = trim(line);
          if (line.empty())
            continue;
          if (line.rfind("subsection", 0) == 0)
            {
              const std::string name = trim(line.substr(10));
              if (!stack.empty())
                throw std::runtime_error("line " + std::to_string(lineno) + ": nested subsections are not declared");
              if (!declared.count(name))
                throw std::runtime_error("line " + std::to_string(lineno) + ": unknown subsection '" + name + "'");
              stack.push_back(name);
            }
          else if (line == "end")
            {
              if (stack.empty())
                throw std::runtime_error("line " + std::to_string(lineno) + ": 'end' without subsection");
              stack.pop_back();
            }
          else if (line.rfind("set", 0) == 0)
            {
              const size_t eq = line.find('=');
              if (eq == std::string::npos)
                throw std::runtime_error("line " + std::to_string(lineno) + ": expected 'set key = value'");
              const std::string key = trim(line.substr(3, eq - 3));
              const std::string val = trim(line.substr(eq + 1));
              const std::string sec = stack.empty() ? "" : stack.back();
              if (!declared[sec].count(key))
                throw std::runtime_error("line " + std::to_string(lineno) + ": unknown entry '" + key +
                                         "' in subsection '" + sec + "'");
              values[sec + "/" + key] = val;
            }
          else
            throw std::runtime_error("line " + std::to_string(lineno) + ": cannot parse '" + line + "'");
        }
      if (!stack.empty())
        throw std::runtime_error("missing 'end' of subsection '" + stack.back() + "'");
    }

    std::string
    get(const std::string &section, const std::string &key) const
    {
      auto it = values.find(section + "/" + key);
      if (it != values.end())
        return it->second;
      auto s = declared.find(section);
      if (s == declared.end() || !s->second.count(key))
        throw std::runtime_error("undeclared entry " + section + "/" + key);
      return s->second.at(key);
    }

    double
    get_double(const std::string &s, const std::string &k) const
    {
      return std::stod(get(s, k));
    }

    int
    get_int(const std::string &s, const std::string &k) const
    {
      return std::stoi(get(s, k));
    }

    bool
    get_bool(const std::string &s, const std::string &k) const
    {
      const std::string v = get(s, k);
      if (v == "true" || v == "1" || v == "yes")
        return true;
      if (v == "false" || v == "0" || v == "no")
        return false;
      throw std::runtime_error("entry " + s + "/" + k + " is not a bool: " + v);
    }

    std::vector<double>
    get_list(const std::string &s, const std::string &k) const
    {
      std::vector<double> r;
      std::string         v = get(s, k);
      for (char &c : v)
        if (c == ',')
          c = ' ';
      std::istringstream is(v);
      double             x;
      while (is >> x)
        r.push_back(x);
      return r;
    }
  };

  // the entries shared by the solid and heat executables
  inline void
  declare_common(Prm &p)
  {
    p.declare("Finite element system", "Polynomial degree", "2");
    p.declare("Finite element system", "Quadrature order", "3");
    p.declare("Geometry", "Global refinement", "0");
    p.declare("Geometry", "Dimension", "2");
    p.declare("Geometry", "Testcase", "turek_hron");
    p.declare("Output", "Output folder", "");
    p.declare("Output", "Output solution", "true");
    p.declare("Output", "Output points", "0,0,0");
    p.declare("Output", "Output tick", "0.1");
    p.declare("Time", "End time", "1");
    p.declare("Time", "Time step size", "0.1");
    for (const char *k : {"precice config-file", "Participant name", "Mesh name", "Read mesh name",
                          "Write mesh name", "Write quadrature index", "Write data specification",
                          "Read data name", "Write data name"})
      p.declare("precice configuration", k, "default");
    // device options (absent from the reference's files; defaults apply)
    p.declare("GPU", "Device", "0");
    p.declare("GPU", "MG precision", "32");
    p.declare("GPU", "FP64 coarse solve", "false");
    p.declare("GPU", "FP64 emulation", "false");
    p.declare("GPU", "CUDA graphs", "true");
    p.declare("GPU", "Dense coarse operator", "true");
  }

  inline void
  declare_solid(Prm &p)
  {
    declare_common(p);
    p.declare("Material properties", "Poisson's ratio", "0.4");
    p.declare("Material properties", "Shear modulus", "0.5e6");
    p.declare("Material properties", "Density", "1000");
    p.declare("Material properties", "Formulation", "1");
    p.declare("Linear solver", "Residual", "1e-6");
    p.declare("Linear solver", "Max iteration multiplier", "1");
    p.declare("Linear solver", "Preconditioner type", "jacobi");
    p.declare("Linear solver", "Preconditioner relaxation", "0.65");
    p.declare("Linear solver", "Estimate condition number", "true");
    p.declare("Linear solver", "Condition number CG iterations", "20");
    p.declare("Linear solver", "MF caching", "scalar_referential");
    p.declare("Linear solver", "MF Chebyshev number CG iterations", "30");
    p.declare("Linear solver", "MF Chebyshev coarse", "true");
    p.declare("Linear solver", "MF Chebyshev coarse accurate eigenvalues", "true");
    p.declare("Nonlinear solver", "Max iterations Newton-Raphson", "10");
    p.declare("Nonlinear solver", "Tolerance force", "1e-9");
    p.declare("Nonlinear solver", "Absolute tolerance force", "0");
    p.declare("Nonlinear solver", "Tolerance displacement", "1e-6");
    p.declare("Nonlinear solver", "Absolute tolerance displacement", "0");
    p.declare("GPU", "Traction", "");
  }
} // namespace mfapp
