/* Force-included before every reference translation unit by the oracle's
 * reference build.  include/barrier.h defines plain C99 `inline` functions
 * (which emit no external definition) and uses the icc-only __declspec;
 * both are neutralised here so gcc can compile and link the sources as they
 * are.  Oracle build support, not product code. */
#define inline static inline
#define __declspec(x)

/* Hooks used by the patched copies (see oracle/build_ref.py). */
extern int gbref_log_buckets;
extern double gbref_cap_mult;
#define GBREF_REQ_CAP(gs) ((long long)(gbref_cap_mult * (double)(gs)->e_size) + 2 * (gs)->v_size + 1024)
