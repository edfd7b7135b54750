// Launch shapes chosen by the autotuner (tuning.cpp reads molds_gb300/tuning.txt).
#pragma once

namespace nddo {

int tuned_groups(int n_mol);            // concurrent molecule groups of a fixed batch
int tuned_tridiag_threads(int n);       // threads of a tridiagonalisation CTA for basis n
int tuned_check_block();                // SCF iterations enqueued per convergence check
int tuned_vec_pairs(int n);             // eigenpairs per CTA of the tridiagonal eigenvector kernel for basis n
bool tuned_vec_smem(int n);             // that kernel's inverse-iteration factors in shared memory (when they fit)

}  // namespace nddo
