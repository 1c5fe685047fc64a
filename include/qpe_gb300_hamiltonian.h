/*
 * qpe_gb300_hamiltonian.h - C ABI of the host-side Hamiltonian term compiler.
 *
 * This is the producer side of the boundary: it turns one- and two-body integrals
 * into the segmented, spin-indexed terms and their exponentiated coefficients that
 * qpe_time_evolve_over_terms / qpe_program_create consume. It follows the
 * reference's Hamiltonian class (cpp/hamiltonian.hpp:24-184, cpp/hamiltonian.cc)
 * term for term, so that a caller without the reference sources gets the same term
 * lists, in the same order, with the same coefficients. Host code only; no GPU.
 */
#ifndef QPE_GB300_HAMILTONIAN_H_
#define QPE_GB300_HAMILTONIAN_H_

#include <stddef.h>
#include <stdint.h>

#include "qpe_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qpe_hamiltonian qpe_hamiltonian;

/* Hamiltonian() (cpp/hamiltonian.hpp:29). */
int qpe_ham_create(qpe_hamiltonian** out);
int qpe_ham_destroy(qpe_hamiltonian* h);

/* AddOneBodyTerm({p, q}, coeff) (cpp/hamiltonian.cc:301-323): 1-based spatial
 * orbitals, p >= q; zero coefficients are ignored. */
int qpe_ham_add_one_body(qpe_hamiltonian* h, int p, int q, double coeff);

/* AddTwoBodyTerm({p, q, r, s}, coeff) (cpp/hamiltonian.cc:325-398): the 8-fold
 * permutations, both spin assignments and the canonical reordering with the 1/2
 * and 1/4 factors. A Broombridge row [i, l, j, k, v] is AddTwoBodyTerm(i, j, k, l). */
int qpe_ham_add_two_body(qpe_hamiltonian* h, int p, int q, int r, int s, double coeff);

/* IngestBroombridge(path, precision) (cpp/hamiltonian.cc:8-144): adds the file's
 * one- and two-body terms, sets the identity term, the orbital count (the largest
 * index in the file) and the electrons per spin (from the first initial-state
 * suggestion), and, if block0 is given (capacity in complex elements), writes
 * that suggestion with its Jordan-Wigner signs as block 0 of the register
 * (C(M, e)^2 interleaved complex doubles, unscaled). Call IndexTerms afterwards. */
int qpe_ham_ingest_broombridge(qpe_hamiltonian* h, const char* path, uint32_t* num_orbitals,
                               uint32_t* num_occupied, double* block0, size_t cap);

/* Fields IngestBroombridge sets from the file (cpp/hamiltonian.cc:13-36, :113-115). */
int qpe_ham_set_num_orbitals(qpe_hamiltonian* h, uint32_t num_orbitals);
/* SetNumOccupied (cpp/hamiltonian.hpp:69): electrons per spin. */
int qpe_ham_set_num_occupied(qpe_hamiltonian* h, uint32_t num_occupied);
int qpe_ham_set_identity(qpe_hamiltonian* h, double identity);
/* SetTimestep (cpp/hamiltonian.hpp:68). */
int qpe_ham_set_timestep(qpe_hamiltonian* h, double t);

int qpe_ham_get_num_orbitals(const qpe_hamiltonian* h, uint32_t* out);
int qpe_ham_get_num_occupied(const qpe_hamiltonian* h, uint32_t* out);
int qpe_ham_get_identity(const qpe_hamiltonian* h, double* out); /* GetIdentityTerm */

/* IndexTerms(SpinIndex::HalfUp) (cpp/hamiltonian.cc:160-197). */
int qpe_ham_index_terms(qpe_hamiltonian* h);

/* Term counts of PrintIndexedSegmentedHamiltonianTerms (cpp/hamiltonian.cc:253-299),
 * in the order pp, pq, pqqp, pqqr, pqrs. */
int qpe_ham_segment_counts(const qpe_hamiltonian* h, size_t counts[5]);

/* Fills one segment (QPE_TERM_* kind) in map order: indices plus the coefficient
 * getters evaluated at the current timestep (pp_term, pq_term(.., 0/1), pqqp_term,
 * pqqr_term(.., 0/1), pqrs_term(.., 0/1); cpp/hamiltonian.cc:661-783). raw, if not
 * NULL, receives the indexed integral value of each term. */
int qpe_ham_segment_terms(const qpe_hamiltonian* h, int kind, qpe_term* out, double* raw, size_t cap);

/* The coefficient getters themselves (cpp/hamiltonian.cc:661-783); out holds
 * interleaved (re, im) pairs: 1 complex for pp/pqqp, 4 for the 2x2 getters. */
int qpe_ham_pp_term(const qpe_hamiltonian* h, uint32_t p, double out[2]);
int qpe_ham_pq_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, uint32_t parity, double out[8]);
int qpe_ham_pqqp_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, double out[2]);
int qpe_ham_pqqr_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, uint32_t r, uint32_t parity,
                      double out[8]);
int qpe_ham_pqrs_term(const qpe_hamiltonian* h, uint32_t p, uint32_t q, uint32_t r, uint32_t s,
                      uint32_t parity, double out[8]);

#ifdef __cplusplus
}
#endif
#endif /* QPE_GB300_HAMILTONIAN_H_ */
