// oomph_ref_driver.cc -- runs the reference's own oomph-lib core on the
// meshes and restated weak forms of the oracle, to pin the C restatement
// (oracle/fe_oracle.c) against the reference's code:
//   * oomph's Gauss<2,3>, TGauss<2,3>, Gauss<3,3> rules and the QElement /
//     TElement shape functions (mode "tables");
//   * oomph's Node/Data equation numbering (Mesh::assign_global_eqn_numbers)
//     and Problem::get_jacobian with the default vectors-of-pairs sparse
//     assembler, zero filter and first-insertion column order
//     (problem.cc:4038-4165, 5332-5666) (mode "assemble").
// The element integrands are written here with oomph's own
// dshape_eulerian_at_knot (the classic oomph route), not the metric-tensor
// route of pyoomph; values therefore agree with the oracle to rounding.
//
// Build: make -C oracle/ref (needs the reference tree; outputs oracle/_ref/).
// TEST INFRASTRUCTURE ONLY.
#include "generic.h"
#include "Telements.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace oomph;

// The vendored oomph-lib calls back into the pyoomph module for SuperLU;
// the driver never solves, so these only satisfy the linker.
extern "C" {
int superlu(int*, int*, int*, int*, double*, int*, int*, double*, int*, int*, int*, void*, int*)
{
  std::fprintf(stderr, "oomph_ref_driver: linear solve not supported\n");
  std::abort();
}
}

namespace
{
enum { Q2_QUAD = 0, P2_TRI = 1, Q2_HEX = 2 };
enum { EQ_POISSON = 0, EQ_NS_TH = 1, EQ_NLDIFF = 2 };

double gauss_source(const std::vector<double>& params, unsigned dim, const Vector<double>& x)
{
  int ng = (int)params[0];
  const double* p = params.data() + 1;
  double f = 0.0;
  for (int k = 0; k < ng; k++)
  {
    double r2 = 0.0;
    for (unsigned i = 0; i < dim; i++)
    {
      double d = x[i] - p[i];
      r2 += d * d;
    }
    double w = p[dim], A = p[dim + 1];
    f += A * std::exp(-r2 / (2.0 * w * w));
    p += dim + 2;
  }
  return f;
}

template<class GEOM>
class RefElement : public virtual GEOM
{
public:
  int Eq = 0;
  unsigned Dim = 2;
  const std::vector<double>* Params = nullptr;

  void fill_in_contribution_to_residuals(Vector<double>& residuals)
  {
    DenseMatrix<double> dummy;
    fill(residuals, dummy, 0);
  }
  void fill_in_contribution_to_jacobian(Vector<double>& residuals, DenseMatrix<double>& jac)
  {
    fill(residuals, jac, 1);
  }

private:
  void fill(Vector<double>& R, DenseMatrix<double>& J, int flag)
  {
    const unsigned nn = this->nnode();
    const unsigned nq = this->integral_pt()->nweight();
    Shape psi(nn);
    DShape dpsidx(nn, Dim);
    for (unsigned ipt = 0; ipt < nq; ipt++)
    {
      const double w = this->integral_pt()->weight(ipt);
      const double Jac = this->dshape_eulerian_at_knot(ipt, psi, dpsidx);
      const double W = w * Jac;
      Vector<double> x(Dim, 0.0);
      for (unsigned l = 0; l < nn; l++)
        for (unsigned i = 0; i < Dim; i++) x[i] += this->nodal_position(l, i) * psi[l];
      if (Eq == EQ_POISSON || Eq == EQ_NLDIFF)
      {
        double u = 0.0, gu[3] = {0, 0, 0};
        for (unsigned l = 0; l < nn; l++)
        {
          u += this->nodal_value(l, 0) * psi[l];
          for (unsigned i = 0; i < Dim; i++) gu[i] += this->nodal_value(l, 0) * dpsidx(l, i);
        }
        const double k = (Eq == EQ_NLDIFF) ? 1.0 + u * u : 1.0;
        const double f = gauss_source(*Params, Dim, x);
        for (unsigned lt = 0; lt < nn; lt++)
        {
          int ie = this->nodal_local_eqn(lt, 0);
          if (ie < 0) continue;
          double gg = 0.0;
          for (unsigned i = 0; i < Dim; i++) gg += gu[i] * dpsidx(lt, i);
          R[ie] += (k * gg - f * psi[lt]) * W;
          if (!flag) continue;
          for (unsigned ls = 0; ls < nn; ls++)
          {
            int je = this->nodal_local_eqn(ls, 0);
            if (je < 0) continue;
            double gs = 0.0;
            for (unsigned i = 0; i < Dim; i++) gs += dpsidx(ls, i) * dpsidx(lt, i);
            double c = k * gs;
            if (Eq == EQ_NLDIFF) c += 2.0 * u * psi[ls] * gg;
            J(ie, je) += c * W;
          }
        }
      }
      else
      {
        // Taylor-Hood: velocity on the six nodes, linear pressure on the
        // three vertices (value index 2).
        const double rho = (*Params)[0], mu = (*Params)[1];
        Vector<double> s(2);
        for (unsigned i = 0; i < 2; i++) s[i] = this->integral_pt()->knot(ipt, i);
        double psi1[3] = {s[0], s[1], 1.0 - s[0] - s[1]};
        DShape dpsi1(3, 2);
        {
          Shape ps(nn);
          DShape dps(nn, 2);
          this->dshape_local(s, ps, dps);
          DenseMatrix<double> inv(2);
          this->local_to_eulerian_mapping(dps, inv);
          DShape d1s(3, 2);
          d1s(0, 0) = 1.0; d1s(0, 1) = 0.0;
          d1s(1, 0) = 0.0; d1s(1, 1) = 1.0;
          d1s(2, 0) = -1.0; d1s(2, 1) = -1.0;
          for (unsigned l = 0; l < 3; l++)
            for (unsigned i = 0; i < 2; i++)
              dpsi1(l, i) = inv(i, 0) * d1s(l, 0) + inv(i, 1) * d1s(l, 1);
        }
        double u[2] = {0, 0}, gu[2][2] = {{0, 0}, {0, 0}}, p = 0.0;
        for (unsigned l = 0; l < nn; l++)
          for (unsigned k = 0; k < 2; k++)
          {
            u[k] += this->nodal_value(l, k) * psi[l];
            for (unsigned i = 0; i < 2; i++) gu[k][i] += this->nodal_value(l, k) * dpsidx(l, i);
          }
        for (unsigned l = 0; l < 3; l++) p += this->nodal_value(l, 2) * psi1[l];
        double tau[2][2], adv[2];
        for (unsigned k = 0; k < 2; k++)
        {
          for (unsigned i = 0; i < 2; i++) tau[k][i] = mu * (gu[k][i] + gu[i][k]) - (k == i ? p : 0.0);
          adv[k] = rho * (u[0] * gu[k][0] + u[1] * gu[k][1]);
        }
        const double divu = gu[0][0] + gu[1][1];
        for (unsigned lt = 0; lt < nn; lt++)
          for (unsigned k = 0; k < 2; k++)
          {
            int ie = this->nodal_local_eqn(lt, k);
            if (ie < 0) continue;
            R[ie] += (tau[k][0] * dpsidx(lt, 0) + tau[k][1] * dpsidx(lt, 1) + adv[k] * psi[lt]) * W;
            if (!flag) continue;
            for (unsigned ls = 0; ls < nn; ls++)
              for (unsigned m = 0; m < 2; m++)
              {
                int je = this->nodal_local_eqn(ls, m);
                if (je < 0) continue;
                double c = 0.0;
                for (unsigned i = 0; i < 2; i++)
                {
                  double dd = 0.0;
                  if (m == k) dd += dpsidx(ls, i);
                  if (m == i) dd += dpsidx(ls, k);
                  c += mu * dd * dpsidx(lt, i);
                }
                double dadv = rho * psi[ls] * gu[k][m];
                if (m == k) dadv += rho * (u[0] * dpsidx(ls, 0) + u[1] * dpsidx(ls, 1));
                c += dadv * psi[lt];
                J(ie, je) += c * W;
              }
            for (unsigned ls = 0; ls < 3; ls++)
            {
              int je = this->nodal_local_eqn(ls, 2);
              if (je < 0) continue;
              J(ie, je) += -psi1[ls] * dpsidx(lt, k) * W;
            }
          }
        for (unsigned lt = 0; lt < 3; lt++)
        {
          int ie = this->nodal_local_eqn(lt, 2);
          if (ie < 0) continue;
          R[ie] += divu * psi1[lt] * W;
          if (!flag) continue;
          for (unsigned ls = 0; ls < nn; ls++)
            for (unsigned m = 0; m < 2; m++)
            {
              int je = this->nodal_local_eqn(ls, m);
              if (je < 0) continue;
              J(ie, je) += dpsidx(ls, m) * psi1[lt] * W;
            }
        }
      }
    }
  }
};

class RefMesh : public Mesh
{
};

class RefProblem : public Problem
{
public:
  RefProblem(Mesh* m, double zero_threshold)
  {
    mesh_pt() = m;
    Numerical_zero_for_sparse_assembly = zero_threshold;
    Sparse_assembly_method = Perform_assembly_using_vectors_of_pairs;
    assign_eqn_numbers();
  }
};

template<class T>
void rd(FILE* f, T* p, size_t n)
{
  if (n && std::fread(p, sizeof(T), n, f) != n)
  {
    std::fprintf(stderr, "short read\n");
    std::exit(2);
  }
}
template<class T>
void wr(FILE* f, const T* p, size_t n)
{
  if (n) std::fwrite(p, sizeof(T), n, f);
}

template<class GEOM>
GeneralisedElement* make_element(int eq, unsigned dim, const std::vector<double>* params)
{
  auto* e = new RefElement<GEOM>();
  e->Eq = eq;
  e->Dim = dim;
  e->Params = params;
  return e;
}

int run_assemble(const char* in_path, const char* out_path)
{
  FILE* f = std::fopen(in_path, "rb");
  if (!f) return 2;
  int32_t hdr[4];
  rd(f, hdr, 4);
  const int etype = hdr[0], eq = hdr[1], dim = hdr[2], nval = hdr[3];
  int64_t sz[2];
  rd(f, sz, 2);
  const int64_t n_nodes = sz[0], n_elem = sz[1];
  int32_t h2[3];
  rd(f, h2, 3);
  const int nne = h2[0], nparams = h2[1], with_jac = h2[2];
  double zero_threshold;
  rd(f, &zero_threshold, 1);
  std::vector<double> x(n_nodes * dim);
  rd(f, x.data(), x.size());
  std::vector<int32_t> conn(n_elem * nne);
  rd(f, conn.data(), conn.size());
  std::vector<int32_t> nvalue(n_nodes);
  rd(f, nvalue.data(), nvalue.size());
  std::vector<int32_t> pinned(n_nodes * nval);
  rd(f, pinned.data(), pinned.size());
  std::vector<double> values(n_nodes * nval);
  rd(f, values.data(), values.size());
  std::vector<double> params(nparams);
  rd(f, params.data(), params.size());
  std::fclose(f);

  RefMesh* mesh = new RefMesh();
  std::vector<Node*> nodes(n_nodes);
  for (int64_t n = 0; n < n_nodes; n++)
  {
    Node* nd = new Node(dim, 1, nvalue[n]);
    for (int i = 0; i < dim; i++) nd->x(i) = x[n * dim + i];
    for (int v = 0; v < nvalue[n]; v++)
    {
      nd->set_value(v, values[n * nval + v]);
      if (pinned[n * nval + v]) nd->pin(v);
    }
    nodes[n] = nd;
    mesh->add_node_pt(nd);
  }
  for (int64_t e = 0; e < n_elem; e++)
  {
    GeneralisedElement* ge;
    if (etype == Q2_QUAD) ge = make_element<QElement<2, 3>>(eq, dim, &params);
    else if (etype == P2_TRI) ge = make_element<TElement<2, 3>>(eq, dim, &params);
    else ge = make_element<QElement<3, 3>>(eq, dim, &params);
    FiniteElement* fe = dynamic_cast<FiniteElement*>(ge);
    for (int j = 0; j < nne; j++) fe->node_pt(j) = nodes[conn[e * nne + j]];
    mesh->add_element_pt(ge);
  }
  RefProblem problem(mesh, zero_threshold);
  const int64_t n_dof = problem.ndof();
  std::vector<int32_t> eqn(n_nodes * nval, -1);
  for (int64_t n = 0; n < n_nodes; n++)
    for (int v = 0; v < nvalue[n]; v++) eqn[n * nval + v] = (int32_t)nodes[n]->eqn_number(v);

  FILE* o = std::fopen(out_path, "wb");
  if (!o) return 3;
  if (with_jac)
  {
    DoubleVector res;
    CRDoubleMatrix jac;
    problem.get_jacobian(res, jac);
    int64_t nnz = jac.nnz();
    int64_t hdro[2] = {n_dof, nnz};
    wr(o, hdro, 2);
    wr(o, eqn.data(), eqn.size());
    std::vector<double> R(n_dof);
    for (int64_t i = 0; i < n_dof; i++) R[i] = res[i];
    wr(o, R.data(), R.size());
    std::vector<int32_t> rp(n_dof + 1);
    for (int64_t i = 0; i <= n_dof; i++) rp[i] = jac.row_start()[i];
    wr(o, rp.data(), rp.size());
    std::vector<int32_t> ci(nnz);
    for (int64_t k = 0; k < nnz; k++) ci[k] = jac.column_index()[k];
    wr(o, ci.data(), ci.size());
    wr(o, jac.value(), nnz);
  }
  else
  {
    DoubleVector res;
    problem.get_residuals(res);
    int64_t hdro[2] = {n_dof, 0};
    wr(o, hdro, 2);
    wr(o, eqn.data(), eqn.size());
    std::vector<double> R(n_dof);
    for (int64_t i = 0; i < n_dof; i++) R[i] = res[i];
    wr(o, R.data(), R.size());
  }
  std::fclose(o);
  return 0;
}

// Writes oomph's integration rules and C2 shape tables at the knots:
// per element type: nq, dim, nnode, then per knot s[dim], w, psi[nnode],
// dpsids[nnode*dim].
int run_tables(const char* out_path)
{
  FILE* o = std::fopen(out_path, "wb");
  if (!o) return 3;
  for (int et = 0; et < 3; et++)
  {
    FiniteElement* fe;
    if (et == Q2_QUAD) fe = new QElement<2, 3>();
    else if (et == P2_TRI) fe = new TElement<2, 3>();
    else fe = new QElement<3, 3>();
    const int32_t nq = fe->integral_pt()->nweight();
    const int32_t dim = fe->dim();
    const int32_t nn = fe->nnode();
    int32_t h[3] = {nq, dim, nn};
    wr(o, h, 3);
    for (int q = 0; q < nq; q++)
    {
      Vector<double> s(dim);
      for (int i = 0; i < dim; i++) s[i] = fe->integral_pt()->knot(q, i);
      double w = fe->integral_pt()->weight(q);
      Shape psi(nn);
      DShape dpsi(nn, dim);
      fe->dshape_local(s, psi, dpsi);
      wr(o, &s[0], dim);
      wr(o, &w, 1);
      for (int l = 0; l < nn; l++) wr(o, &psi[l], 1);
      for (int l = 0; l < nn; l++)
        for (int i = 0; i < dim; i++) wr(o, &dpsi(l, i), 1);
    }
    delete fe;
  }
  std::fclose(o);
  return 0;
}
} // namespace

int main(int argc, char** argv)
{
  if (argc >= 4 && std::strcmp(argv[1], "assemble") == 0) return run_assemble(argv[2], argv[3]);
  if (argc >= 3 && std::strcmp(argv[1], "tables") == 0) return run_tables(argv[2]);
  std::fprintf(stderr, "usage: %s assemble IN OUT | tables OUT\n", argv[0]);
  return 1;
}
