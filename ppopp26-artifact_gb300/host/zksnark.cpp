// zksnark.cpp -- quotient-constraint entry points over libppfr.so.
#include "zksnark.h"

#include <string>

#include "pp_ops.h"

namespace {

uint64_t count_of(SyncedMemory &m, const char *what) {
  if (m.size() % 32) throw pp::Error(PP_E_INVAL, std::string(what) + ": size is not a multiple of 32 bytes");
  return m.size() / 32;
}

// device view of a vector of n elements (scalars: n = 1)
const void *dev(SyncedMemory &m, uint64_t n, cudaStream_t s, const char *what) {
  if (count_of(m, what) < n) throw pp::Error(PP_E_INVAL, std::string(what) + ": buffer too short");
  return m.mutable_gpu_data_async(s);
}

}  // namespace

namespace cuda {

SyncedMemory compute_gate_constraint_allmerge_cuda(
    SyncedMemory a_val, SyncedMemory b_val, SyncedMemory c_val, SyncedMemory d_val,
    SyncedMemory a_next_eval, SyncedMemory b_next_eval, SyncedMemory d_next_eval, SyncedMemory q_m,
    SyncedMemory q_l, SyncedMemory q_r, SyncedMemory q_o, SyncedMemory q_4, SyncedMemory q_c,
    SyncedMemory q_hl, SyncedMemory q_hr, SyncedMemory q_h4, SyncedMemory q_arith,
    SyncedMemory range, SyncedMemory logic, SyncedMemory fixed_group_add,
    SyncedMemory variable_group_add, SyncedMemory pi_eval_8n, SyncedMemory four, SyncedMemory one,
    SyncedMemory two, SyncedMemory three, SyncedMemory kappa_range, SyncedMemory kappa_sq_range,
    SyncedMemory kappa_cu_range, SyncedMemory range_challenge, SyncedMemory P_D, SyncedMemory nine,
    SyncedMemory kappa_cu_logic, SyncedMemory eighteen, SyncedMemory eightyone,
    SyncedMemory eightythree, SyncedMemory kappa_qu_logic, SyncedMemory logic_challenge,
    SyncedMemory P_A, SyncedMemory kappa_fb, SyncedMemory kappa_sq_fb, SyncedMemory kappa_cu_fb,
    SyncedMemory fb_challenge, SyncedMemory kappa_vb, SyncedMemory kappa_sq_vb,
    SyncedMemory vb_challenge, int64_t SBOX_ALPHA, cudaStream_t stream) {
  const char *what = "compute_gate_constraint_allmerge_cuda";
  const uint64_t n = count_of(a_val, what);
  SyncedMemory out(a_val.size());
  SyncedMemory *vec[PP_GATE_NV] = {&a_val, &b_val, &c_val, &d_val, &a_next_eval, &b_next_eval,
                                   &d_next_eval, &q_m, &q_l, &q_r, &q_o, &q_4, &q_c, &q_hl, &q_hr,
                                   &q_h4, &q_arith, &range, &logic, &fixed_group_add,
                                   &variable_group_add, &pi_eval_8n};
  SyncedMemory *sc[PP_GATE_NS] = {&four, &one, &two, &three, &kappa_range, &kappa_sq_range,
                                  &kappa_cu_range, &range_challenge, &P_D, &nine, &kappa_cu_logic,
                                  &eighteen, &eightyone, &eightythree, &kappa_qu_logic,
                                  &logic_challenge, &P_A, &kappa_fb, &kappa_sq_fb, &kappa_cu_fb,
                                  &fb_challenge, &kappa_vb, &kappa_sq_vb, &vb_challenge};
  pp_gate_args a;
  for (int j = 0; j < PP_GATE_NV; ++j) a.v[j] = dev(*vec[j], n, stream, what);
  for (int j = 0; j < PP_GATE_NS; ++j) a.s[j] = dev(*sc[j], 1, stream, what);
  a.sbox_alpha = SBOX_ALPHA;
  void *o = out.mutable_gpu_data_async(stream);
  pp::check(pp_gate_constraint(&a, o, n, stream), what);
  return out;
}

void compute_quotient_identity_range_check_i(SyncedMemory x, SyncedMemory w_l, SyncedMemory w_r,
                                             SyncedMemory w_o, SyncedMemory w_4, SyncedMemory z,
                                             SyncedMemory alpha, SyncedMemory beta,
                                             SyncedMemory gamma, SyncedMemory k1, SyncedMemory k2,
                                             SyncedMemory k3, SyncedMemory result,
                                             cudaStream_t stream) {
  const char *what = "compute_quotient_identity_range_check_i";
  const uint64_t n = count_of(x, what);
  pp_perm_quotient_args a = {};
  a.x = dev(x, n, stream, what);
  SyncedMemory *w[4] = {&w_l, &w_r, &w_o, &w_4};
  for (int j = 0; j < 4; ++j) a.w[j] = dev(*w[j], n, stream, what);
  a.z = dev(z, n, stream, what);
  a.alpha = dev(alpha, 1, stream, what);
  a.beta = dev(beta, 1, stream, what);
  a.gamma = dev(gamma, 1, stream, what);
  a.k[0] = dev(k1, 1, stream, what);
  a.k[1] = dev(k2, 1, stream, what);
  a.k[2] = dev(k3, 1, stream, what);
  void *r = const_cast<void *>(dev(result, n, stream, what));
  pp::check(pp_quotient_identity(&a, r, n, stream), what);
}

void compute_quotient_copy_range_check_i(SyncedMemory left_sigma, SyncedMemory right_sigma,
                                         SyncedMemory out_sigma, SyncedMemory fourth_sigma,
                                         SyncedMemory mod, SyncedMemory w_l, SyncedMemory w_r,
                                         SyncedMemory w_o, SyncedMemory w_4, SyncedMemory z_next,
                                         SyncedMemory alpha, SyncedMemory beta, SyncedMemory gamma,
                                         SyncedMemory result, cudaStream_t stream) {
  const char *what = "compute_quotient_copy_range_check_i";
  const uint64_t n = count_of(left_sigma, what);
  pp_perm_quotient_args a = {};
  SyncedMemory *sg[4] = {&left_sigma, &right_sigma, &out_sigma, &fourth_sigma};
  SyncedMemory *w[4] = {&w_l, &w_r, &w_o, &w_4};
  for (int j = 0; j < 4; ++j) {
    a.sigma[j] = dev(*sg[j], n, stream, what);
    a.w[j] = dev(*w[j], n, stream, what);
  }
  a.mod = dev(mod, n, stream, what);
  a.z_next = dev(z_next, n, stream, what);
  a.alpha = dev(alpha, 1, stream, what);
  a.beta = dev(beta, 1, stream, what);
  a.gamma = dev(gamma, 1, stream, what);
  void *r = const_cast<void *>(dev(result, n, stream, what));
  pp::check(pp_quotient_copy(&a, r, n, stream), what);
}

void compute_quotient_term_check_one_i(SyncedMemory z, SyncedMemory l1, SyncedMemory one,
                                       SyncedMemory result, cudaStream_t stream) {
  const char *what = "compute_quotient_term_check_one_i";
  const uint64_t n = count_of(z, what);
  pp_perm_quotient_args a = {};
  a.z = dev(z, n, stream, what);
  a.l1 = dev(l1, n, stream, what);
  a.one = dev(one, 1, stream, what);
  void *r = const_cast<void *>(dev(result, n, stream, what));
  pp::check(pp_quotient_term_one(&a, r, n, stream), what);
}

}  // namespace cuda
