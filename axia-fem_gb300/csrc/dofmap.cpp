// dofmap.cpp -- the DOF map with multi-point constraints (host side).
//
// The reference's DofMap::build (solver/src/constraint.rs:26-136) turns the
// prescribed displacements and the MPCs (u_slave = sum alpha_m u_m + u0) into
// u = u0 + T x: every DOF that is neither prescribed nor a slave is an
// independent unknown (numbered in ascending DOF order); a slave's row of T
// holds its masters expanded through nested slaves (up to 32 passes), with
// prescribed masters folded into its u0.  The steps and their order are the
// reference's, because T and u0 enter the reduced system bit for bit:
//   * prescribed: the last entry for a DOF wins (analysis.rs:556-565);
//   * an MPC whose slave is out of range or prescribed is ignored; of several
//     MPCs naming the same slave, the last one wins (HashMap::insert);
//   * expansion pass: each term on a slave is replaced by that slave's MPC
//     scaled by the term's alpha (the particular part gains alpha * u0), then
//     the terms are coalesced: stable sort by DOF, equal DOFs summed in
//     order, a DOF starts an entry only with a non-zero alpha, entries with
//     |alpha| <= 1e-16 dropped (constraint.rs:219-235);
//   * after the passes, prescribed masters move into the particular part; a
//     master that is still a slave is a cyclic MPC (an error);
//   * T row: (ind_of[d], 1) for an independent DOF, the non-zero
//     (ind_of[m], alpha) terms for a slave, nothing for a prescribed DOF.
// A master outside [0, ndof) is AXIA_ERR_INVALID_ARG (the reference would
// index out of bounds).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/axia_gpu.h"

struct axia_dofmap {
  int64_t n_full = 0, n_ind = 0;
  std::vector<double> u0;
  std::vector<int64_t> t_ptr, t_col, ind_of;
  std::vector<double> t_val;
};

namespace {

using Term = std::pair<int64_t, double>;

void merge_terms(std::vector<Term>& terms) {
  std::stable_sort(terms.begin(), terms.end(), [](const Term& a, const Term& b) { return a.first < b.first; });
  std::vector<Term> merged;
  merged.reserve(terms.size());
  for (const Term& t : terms) {
    if (!merged.empty() && merged.back().first == t.first)
      merged.back().second += t.second;
    else if (std::fabs(t.second) > 0.0)
      merged.push_back(t);
  }
  terms.clear();
  for (const Term& t : merged)
    if (std::fabs(t.second) > 1e-16) terms.push_back(t);
}

}  // namespace

extern "C" {

int32_t axia_dofmap_build(int64_t ndof, int64_t n_presc, const int64_t* presc_dof, const double* presc_val,
                          int64_t n_mpc, const int64_t* mpc_slave, const int64_t* mpc_ptr, const int64_t* mpc_master,
                          const double* mpc_alpha, const double* mpc_u0, axia_dofmap** out) {
  if (!out || ndof <= 0 || n_presc < 0 || n_mpc < 0) return AXIA_ERR_INVALID_ARG;
  if ((n_presc > 0 && (!presc_dof || !presc_val)) || (n_mpc > 0 && (!mpc_slave || !mpc_ptr || !mpc_u0)))
    return AXIA_ERR_INVALID_ARG;
  *out = nullptr;
  for (int64_t i = 0; i < n_mpc; ++i)
    if (mpc_ptr[i + 1] < mpc_ptr[i]) return AXIA_ERR_INVALID_ARG;
  if (n_mpc > 0 && mpc_ptr[n_mpc] > mpc_ptr[0] && (!mpc_master || !mpc_alpha)) return AXIA_ERR_INVALID_ARG;
  std::vector<char> fixed((size_t)ndof, 0);
  std::vector<double> fixed_val((size_t)ndof, 0.0);
  for (int64_t k = 0; k < n_presc; ++k) {
    const int64_t d = presc_dof[k];
    if (d < 0 || d >= ndof) continue;
    fixed[d] = 1;
    fixed_val[d] = presc_val[k];
  }
  std::vector<int64_t> owner((size_t)ndof, -1);  // the MPC that defines slave d
  for (int64_t i = 0; i < n_mpc; ++i) {
    const int64_t s = mpc_slave[i];
    if (s >= 0 && s < ndof && !fixed[s]) owner[s] = i;
  }
  auto* m = new axia_dofmap();
  m->n_full = ndof;
  m->u0 = fixed_val;
  std::vector<std::vector<Term>> rows((size_t)ndof);
  for (int64_t i = 0; i < n_mpc; ++i) {
    const int64_t s = mpc_slave[i];
    if (s < 0 || s >= ndof || owner[s] != i) continue;
    std::vector<Term> terms;
    for (int64_t q = mpc_ptr[i]; q < mpc_ptr[i + 1]; ++q) terms.emplace_back(mpc_master[q], mpc_alpha[q]);
    double part = mpc_u0[i];
    for (int pass = 0; pass < 32; ++pass) {
      std::vector<Term> next;
      bool expanded = false;
      for (const Term& t : terms) {
        const int64_t k = (t.first >= 0 && t.first < ndof) ? owner[t.first] : -1;
        if (k < 0) {
          next.push_back(t);
          continue;
        }
        expanded = true;
        part += t.second * mpc_u0[k];
        for (int64_t q = mpc_ptr[k]; q < mpc_ptr[k + 1]; ++q) next.emplace_back(mpc_master[q], t.second * mpc_alpha[q]);
      }
      merge_terms(next);
      terms.swap(next);
      if (!expanded) break;
    }
    for (const Term& t : terms) {
      if (t.first < 0 || t.first >= ndof) {
        delete m;
        return AXIA_ERR_INVALID_ARG;
      }
      if (fixed[t.first])
        part += t.second * fixed_val[t.first];
      else if (owner[t.first] >= 0) {
        delete m;
        return AXIA_ERR_INVALID_ARG;  // cyclic MPC (constraint.rs:81)
      } else
        rows[s].push_back(t);
    }
    m->u0[s] = part;
  }
  m->ind_of.assign((size_t)ndof, -1);
  bool any_fixed = false, any_slave = false;
  for (int64_t d = 0; d < ndof; ++d) {
    any_fixed = any_fixed || fixed[d];
    any_slave = any_slave || owner[d] >= 0;
    if (!fixed[d] && owner[d] < 0) m->ind_of[d] = m->n_ind++;
  }
  if (m->n_ind == 0 && !any_slave && !any_fixed) {  // constraint.rs:111-113
    delete m;
    return AXIA_ERR_NO_FREE_DOF;
  }
  m->t_ptr.assign((size_t)ndof + 1, 0);
  for (int64_t d = 0; d < ndof; ++d) {
    if (m->ind_of[d] >= 0) {
      m->t_col.push_back(m->ind_of[d]);
      m->t_val.push_back(1.0);
    } else if (owner[d] >= 0) {
      for (const Term& t : rows[d]) {
        const int64_t col = m->ind_of[t.first];
        if (col >= 0 && std::fabs(t.second) > 0.0) {
          m->t_col.push_back(col);
          m->t_val.push_back(t.second);
        }
      }
    }
    m->t_ptr[d + 1] = (int64_t)m->t_col.size();
  }
  *out = m;
  return AXIA_OK;
}

int64_t axia_dofmap_n_ind(const axia_dofmap* m) { return m ? m->n_ind : -1; }

int64_t axia_dofmap_export(const axia_dofmap* m, int64_t* t_ptr, int64_t* t_col, double* t_val, double* u0,
                           int64_t* ind_of) {
  if (!m) return -1;
  const int64_t nnz = (int64_t)m->t_col.size();
  if (t_ptr) std::copy(m->t_ptr.begin(), m->t_ptr.end(), t_ptr);
  if (t_col) std::copy(m->t_col.begin(), m->t_col.end(), t_col);
  if (t_val) std::copy(m->t_val.begin(), m->t_val.end(), t_val);
  if (u0) std::copy(m->u0.begin(), m->u0.end(), u0);
  if (ind_of) std::copy(m->ind_of.begin(), m->ind_of.end(), ind_of);
  return nnz;
}

void axia_dofmap_free(axia_dofmap* m) { delete m; }

}  // extern "C"

// Accessors for the device side (reduce.cu).
int64_t dofmap_n_full(const axia_dofmap* m) { return m->n_full; }
const int64_t* dofmap_t_ptr(const axia_dofmap* m) { return m->t_ptr.data(); }
const int64_t* dofmap_t_col(const axia_dofmap* m) { return m->t_col.data(); }
const double* dofmap_t_val(const axia_dofmap* m) { return m->t_val.data(); }
const double* dofmap_u0(const axia_dofmap* m) { return m->u0.data(); }
int64_t dofmap_t_nnz(const axia_dofmap* m) { return (int64_t)m->t_col.size(); }
