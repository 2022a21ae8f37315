// oomph_hang_driver.cc -- runs the reference's own oomph-lib refinement
// machinery on the oracle's Q2 meshes, to pin the hanging-node restatement
// (oracle/hang_oracle.py) and the package's refined meshes against it:
//   * quadtree refinement by RefineableQElement<2>::build and
//     TreeBasedRefineableMeshBase::refine_selected_elements / adapt_mesh:
//     the leaves' order, the new nodes, and Mesh::reorder_nodes (first
//     encounter over the elements) after every adapt;
//   * hanging nodes by RefineableQElement<2>::setup_hang_for_value and
//     their completion by complete_hanging_nodes (masters of masters,
//     weights multiplied, merged in a map keyed by the node's address);
//   * equation numbering with constrained hanging values, and
//     Problem::get_jacobian with the vectors-of-pairs assembler, the
//     element's hanging rows and columns going to their masters' equations
//     (local_hang_eqn), as pyoomph's jitbridge_hang.h master loops do.
// The element integrand is the Poisson form of oracle/fe_oracle.c written
// with oomph's dshape_eulerian_at_knot; only the refinement, numbering and
// assembly machinery is the reference's.
//
// Build: make -C oracle/ref (needs the reference tree; outputs oracle/_ref/).
// TEST INFRASTRUCTURE ONLY.
#include "generic.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>

using namespace oomph;

extern "C" {
int superlu(int*, int*, int*, int*, double*, int*, int*, double*, int*, int*, int*, void*, int*)
{
  std::fprintf(stderr, "oomph_hang_driver: linear solve not supported\n");
  std::abort();
}
}

namespace
{
std::vector<double> Params;   // [ng, (cx, cy, w, A) * ng]

double gauss_source(const Vector<double>& x)
{
  const int ng = (int)Params[0];
  const double* p = Params.data() + 1;
  double f = 0.0;
  for (int k = 0; k < ng; k++)
  {
    const double d0 = x[0] - p[0], d1 = x[1] - p[1];
    const double w = p[2], A = p[3];
    f += A * std::exp(-(d0 * d0 + d1 * d1) / (2.0 * w * w));
    p += 4;
  }
  return f;
}

// Q2 quad with one continuously interpolated value, refineable by quadtrees
class HangElement : public virtual QElement<2, 3>, public virtual RefineableQElement<2>
{
public:
  HangElement() : QElement<2, 3>(), RefineableQElement<2>() {}

  unsigned required_nvalue(const unsigned& n) const
  {
    return 1;
  }
  unsigned ncont_interpolated_values() const
  {
    return 1;
  }
  void get_interpolated_values(const unsigned& t, const Vector<double>& s, Vector<double>& values)
  {
    values.resize(1);
    Shape psi(9);
    shape(s, psi);
    values[0] = 0.0;
    for (unsigned l = 0; l < 9; l++) values[0] += nodal_value(t, l, 0) * psi[l];
  }
  void rebuild_from_sons(Mesh*& mesh_pt) {}
  void check_integrity(double& max_error)
  {
    max_error = 0.0;
  }
  void further_setup_hanging_nodes() {}
  unsigned nvertex_node() const
  {
    return QElement<2, 3>::nvertex_node();
  }
  Node* vertex_node_pt(const unsigned& j) const
  {
    return QElement<2, 3>::vertex_node_pt(j);
  }

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
  // local equations (and weights) of nodal value 0 of node l: its own, or
  // its masters' if it hangs
  void eqns(unsigned l, std::vector<int>& eq, std::vector<double>& w)
  {
    eq.clear();
    w.clear();
    Node* nod = node_pt(l);
    if (nod->is_hanging(0))
    {
      HangInfo* h = nod->hanging_pt(0);
      for (unsigned m = 0; m < h->nmaster(); m++)
      {
        eq.push_back(local_hang_eqn(h->master_node_pt(m), 0));
        w.push_back(h->master_weight(m));
      }
    }
    else
    {
      eq.push_back(nodal_local_eqn(l, 0));
      w.push_back(1.0);
    }
  }

  void fill(Vector<double>& R, DenseMatrix<double>& J, int flag)
  {
    const unsigned nn = 9, nq = integral_pt()->nweight();
    Shape psi(nn);
    DShape dpsidx(nn, 2);
    std::vector<int> ei, ej;
    std::vector<double> wi, wj;
    for (unsigned ipt = 0; ipt < nq; ipt++)
    {
      const double W = integral_pt()->weight(ipt) * dshape_eulerian_at_knot(ipt, psi, dpsidx);
      Vector<double> x(2, 0.0);
      double gu[2] = {0.0, 0.0};
      for (unsigned l = 0; l < nn; l++)
      {
        const double u = nodal_value(l, 0);   // hanging nodes: interpolated from the masters
        for (unsigned i = 0; i < 2; i++)
        {
          x[i] += nodal_position(l, i) * psi[l];
          gu[i] += u * dpsidx(l, i);
        }
      }
      const double f = gauss_source(x);
      for (unsigned lt = 0; lt < nn; lt++)
      {
        eqns(lt, ei, wi);
        const double gg = gu[0] * dpsidx(lt, 0) + gu[1] * dpsidx(lt, 1);
        for (unsigned a = 0; a < ei.size(); a++)
        {
          if (ei[a] < 0) continue;
          R[ei[a]] += (gg - f * psi[lt]) * W * wi[a];
          if (!flag) continue;
          for (unsigned ls = 0; ls < nn; ls++)
          {
            eqns(ls, ej, wj);
            const double gs = dpsidx(ls, 0) * dpsidx(lt, 0) + dpsidx(ls, 1) * dpsidx(lt, 1);
            for (unsigned b = 0; b < ej.size(); b++)
            {
              if (ej[b] < 0) continue;
              J(ei[a], ej[b]) += gs * W * wi[a] * wj[b];
            }
          }
        }
      }
    }
  }
};

class HangMesh : public virtual TreeBasedRefineableMesh<HangElement>
{
public:
  void setup_tree_forest()
  {
    Vector<TreeRoot*> roots;
    for (unsigned e = 0; e < nelement(); e++)
      roots.push_back(new QuadTreeRoot(dynamic_cast<RefineableElement*>(element_pt(e))));
    Forest_pt = new QuadTreeForest(roots);
  }
};

class HangProblem : public Problem
{
public:
  explicit HangProblem(Mesh* m)
  {
    mesh_pt() = m;
    Numerical_zero_for_sparse_assembly = -1.0;   // keep every structural entry
    Sparse_assembly_method = Perform_assembly_using_vectors_of_pairs;
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

// input: int32 n_nodes, n_elem, n_refine, n_params; float64 x[n_nodes*2];
// int32 conn[n_elem*9]; uint32 bmask[n_nodes]; float64 refine[n_refine*3]
// (level, centre x, centre y of the elements to split); float64
// params[n_params]; float64 dofs of the refined mesh follow in a second
// file (the values; see run)
int run(const char* in_path, const char* dofs_path, const char* out_path)
{
  FILE* f = std::fopen(in_path, "rb");
  if (!f) return 2;
  int32_t hdr[4];
  rd(f, hdr, 4);
  const int n_nodes = hdr[0], n_elem = hdr[1], n_refine = hdr[2], n_params = hdr[3];
  std::vector<double> x(2 * (size_t)n_nodes), refine(3 * (size_t)n_refine);
  std::vector<int32_t> conn(9 * (size_t)n_elem);
  std::vector<uint32_t> bmask(n_nodes);
  rd(f, x.data(), x.size());
  rd(f, conn.data(), conn.size());
  rd(f, bmask.data(), bmask.size());
  rd(f, refine.data(), refine.size());
  Params.resize(n_params);
  rd(f, Params.data(), Params.size());
  std::fclose(f);

  QuadTree::setup_static_data();          // the quadtrees' direction tables (oomph's meshes call it first)
  HangMesh* mesh = new HangMesh;
  mesh->set_nboundary(4);
  // nodes created in the template's node order (as pyoomph generates a mesh
  // from its template), each by the first element that holds it
  std::vector<HangElement*> els(n_elem);
  for (int e = 0; e < n_elem; e++) els[e] = new HangElement;
  std::vector<int> first_e(n_nodes, -1), first_j(n_nodes, -1);
  for (int e = 0; e < n_elem; e++)
    for (unsigned j = 0; j < 9; j++)
    {
      const int g = conn[9 * e + j];
      if (first_e[g] < 0)
      {
        first_e[g] = e;
        first_j[g] = (int)j;
      }
    }
  std::vector<Node*> nodes(n_nodes, nullptr);
  for (int g = 0; g < n_nodes; g++)
  {
    HangElement* el = els[first_e[g]];
    const unsigned j = (unsigned)first_j[g];
    nodes[g] = bmask[g] ? el->construct_boundary_node(j) : el->construct_node(j);
    nodes[g]->x(0) = x[2 * g];
    nodes[g]->x(1) = x[2 * g + 1];
  }
  for (int e = 0; e < n_elem; e++)
  {
    for (unsigned j = 0; j < 9; j++) els[e]->node_pt(j) = nodes[conn[9 * e + j]];
    mesh->add_element_pt(els[e]);
  }
  for (int g = 0; g < n_nodes; g++)
  {
    mesh->add_node_pt(nodes[g]);
    for (unsigned b = 0; b < 4; b++)
      if (bmask[g] & (1u << b)) mesh->add_boundary_node(b, nodes[g]);
    if (bmask[g]) nodes[g]->pin(0);        // u = 0 on the outer boundary
  }
  mesh->setup_boundary_element_info();      // which element edges lie on which boundary (refinement reads it)
  mesh->setup_tree_forest();
  // level by level: split the leaves of that level whose centre is listed
  unsigned max_level = 0;
  for (int k = 0; k < n_refine; k++) max_level = std::max(max_level, (unsigned)refine[3 * k]);
  for (unsigned level = 0; level <= max_level; level++)
  {
    Vector<unsigned> sel;
    for (unsigned e = 0; e < mesh->nelement(); e++)
    {
      RefineableElement* el = dynamic_cast<RefineableElement*>(mesh->element_pt(e));
      if (el->refinement_level() != level) continue;
      Node* c = mesh->finite_element_pt(e)->node_pt(4);
      for (int k = 0; k < n_refine; k++)
        if ((unsigned)refine[3 * k] == level && std::fabs(refine[3 * k + 1] - c->x(0)) < 1e-12 &&
            std::fabs(refine[3 * k + 2] - c->x(1)) < 1e-12)
        {
          sel.push_back(e);
          break;
        }
    }
    if (!sel.empty()) mesh->refine_selected_elements(sel);
  }
  HangProblem problem(mesh);
  problem.assign_eqn_numbers();

  const unsigned nn = mesh->nnode(), ne = mesh->nelement();
  std::map<Node*, int> idx;
  for (unsigned i = 0; i < nn; i++) idx[mesh->node_pt(i)] = (int)i;
  // values of the free dofs from the dofs file (f64 per equation), if given
  const unsigned long ndof = problem.ndof();
  if (dofs_path && dofs_path[0])
  {
    FILE* g = std::fopen(dofs_path, "rb");
    if (!g) return 2;
    std::vector<double> d(ndof);
    rd(g, d.data(), d.size());
    std::fclose(g);
    for (unsigned i = 0; i < nn; i++)
    {
      const long q = mesh->node_pt(i)->eqn_number(0);
      if (q >= 0) mesh->node_pt(i)->set_value(0, d[q]);
    }
  }
  DoubleVector R;
  CRDoubleMatrix J;
  problem.get_jacobian(R, J);

  FILE* o = std::fopen(out_path, "wb");
  if (!o) return 2;
  int32_t ohdr[4] = {(int32_t)nn, (int32_t)ne, (int32_t)ndof, (int32_t)J.nnz()};
  wr(o, ohdr, 4);
  for (unsigned i = 0; i < nn; i++)
  {
    const double p[2] = {mesh->node_pt(i)->x(0), mesh->node_pt(i)->x(1)};
    wr(o, p, 2);
  }
  for (unsigned e = 0; e < ne; e++)
    for (unsigned j = 0; j < 9; j++)
    {
      const int32_t k = idx[mesh->finite_element_pt(e)->node_pt(j)];
      wr(o, &k, 1);
    }
  for (unsigned i = 0; i < nn; i++)
  {
    const int32_t q = (int32_t)mesh->node_pt(i)->eqn_number(0);
    wr(o, &q, 1);
  }
  for (unsigned i = 0; i < nn; i++)
  {
    Node* nod = mesh->node_pt(i);
    int32_t nm = 0;
    if (nod->is_hanging(0)) nm = (int32_t)nod->hanging_pt(0)->nmaster();
    wr(o, &nm, 1);
    for (int32_t m = 0; m < nm; m++)
    {
      const int32_t k = idx[nod->hanging_pt(0)->master_node_pt(m)];
      const double w = nod->hanging_pt(0)->master_weight(m);
      wr(o, &k, 1);
      wr(o, &w, 1);
    }
  }
  wr(o, J.row_start(), ndof + 1);
  wr(o, J.column_index(), J.nnz());
  wr(o, J.value(), J.nnz());
  for (unsigned long i = 0; i < ndof; i++)
  {
    const double r = R[i];
    wr(o, &r, 1);
  }
  std::fclose(o);
  return 0;
}
} // namespace

int main(int argc, char** argv)
{
  if (argc < 4)
  {
    std::fprintf(stderr, "usage: oomph_hang_driver in.bin dofs.bin|'' out.bin\n");
    return 1;
  }
  return run(argv[1], argv[2], argv[3]);
}
