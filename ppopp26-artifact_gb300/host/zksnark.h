// zksnark.h -- the reference's PLONK quotient-constraint entry points
// (PLONK/utils/zkp/cuda/zksnark.cuh:103-127, namespace cuda), same names,
// argument order and buffer conventions, forwarding to libppfr.so:
//
//   zksnark_comute_gate_constraint.cu:30        compute_gate_constraint_allmerge_cuda
//   zksnark_compute_permutation_constraint.cu:49 compute_quotient_identity_range_check_i
//   zksnark_compute_permutation_constraint.cu:80 compute_quotient_copy_range_check_i
//   zksnark_compute_permutation_constraint.cu:113 compute_quotient_term_check_one_i
//
// Every argument is a SyncedMemory of n Fr (vectors) or one Fr (scalars);
// n is taken from the first vector, as the reference does.  Errors throw
// pp::Error (the reference has no error path).
#pragma once
#include <cstdint>

#include "syncedmem.h"

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
    SyncedMemory vb_challenge, int64_t SBOX_ALPHA, cudaStream_t stream = (cudaStream_t)0);

void compute_quotient_identity_range_check_i(SyncedMemory x, SyncedMemory w_l, SyncedMemory w_r,
                                             SyncedMemory w_o, SyncedMemory w_4, SyncedMemory z,
                                             SyncedMemory alpha, SyncedMemory beta,
                                             SyncedMemory gamma, SyncedMemory k1, SyncedMemory k2,
                                             SyncedMemory k3, SyncedMemory result,
                                             cudaStream_t stream = (cudaStream_t)0);

void compute_quotient_copy_range_check_i(SyncedMemory left_sigma, SyncedMemory right_sigma,
                                         SyncedMemory out_sigma, SyncedMemory fourth_sigma,
                                         SyncedMemory mod, SyncedMemory w_l, SyncedMemory w_r,
                                         SyncedMemory w_o, SyncedMemory w_4, SyncedMemory z_next,
                                         SyncedMemory alpha, SyncedMemory beta, SyncedMemory gamma,
                                         SyncedMemory result,
                                         cudaStream_t stream = (cudaStream_t)0);

void compute_quotient_term_check_one_i(SyncedMemory z, SyncedMemory l1, SyncedMemory one,
                                       SyncedMemory result, cudaStream_t stream = (cudaStream_t)0);

}  // namespace cuda
