/*
 * wfa_oracle_bialign.c -- CPU restatement of WFA2-lib's BiWFA (ultralow memory
 * mode).  TEST INFRASTRUCTURE ONLY (see wfa_oracle.h).
 *
 * Placeholder until the breakpoint restatement lands: it answers ultralow
 * requests with the unidirectional alignment, whose SCORE equals BiWFA's
 * (tests/wfa.utest.sh:79-90 compares the two on score only) but whose CIGAR
 * can differ on ties.  Tests therefore check ultralow on score only.
 */
#include "wfa_oracle_internal.h"

void oracle_bialign(const pen_t* p, const char* P, int plen, const char* T, int tlen,
                    oracle_ws_t* ws, int32_t* out_score, int32_t* out_status, char* ops,
                    int32_t* ops_len) {
  oracle_align_one(ws, p, P, plen, T, tlen, out_score, out_status, ops, ops_len, NULL, NULL);
}
