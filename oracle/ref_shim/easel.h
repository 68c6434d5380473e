/* Minimal stand-in for the Easel library header, written for this project.
 *
 * Easel is not shipped with the Infernal source tree this project studies,
 * so the reference scanner sources (cm_dpsearch.c, cm_dpsearch_trunc.c,
 * cm_mx.c, logsum.c, cm_tophits.c, cm_trunc.c) are compiled against this
 * shim to serve as the parity checker.  Only the handful of types, macros
 * and functions that those files touch are declared; structures that the
 * scanners never dereference are left opaque.
 */
#ifndef INFGB_SHIM_EASEL_H
#define INFGB_SHIM_EASEL_H
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <inttypes.h>
#include <float.h>
#include <assert.h>

typedef uint8_t ESL_DSQ;

#define eslOK              0
#define eslFAIL            1
#define eslEOL             2
#define eslEOF             3
#define eslEOD             4
#define eslEMEM            5
#define eslENOTFOUND       6
#define eslEFORMAT         7
#define eslEAMBIGUOUS      8
#define eslEDIVZERO        9
#define eslEINCOMPAT      10
#define eslEINVAL         11
#define eslESYS           12
#define eslECORRUPT       13
#define eslEINCONCEIVABLE 14
#define eslESYNTAX        15
#define eslERANGE         16
#define eslEDUP           17
#define eslENOHALT        18
#define eslENORESULT      19
#define eslENODATA        20
#define eslETYPE          21
#define eslEOVERWRITE     22
#define eslENOSPACE       23
#define eslEUNIMPLEMENTED 24
#define eslENOFORMAT      25
#define eslENOALPHABET    26
#define eslEWRITE         27
#define eslEINACCURATE    28

#define eslERRBUFSIZE 128
#define eslINFINITY   INFINITY
#define eslCONST_LOG2 0.69314718055994529
#ifndef TRUE
#define TRUE  1
#define FALSE 0
#endif

#define ESL_MIN(a,b) (((a)<(b))?(a):(b))
#define ESL_MAX(a,b) (((a)>(b))?(a):(b))

#define ESL_ALLOC(p, size) do { \
    if (((p) = malloc(size)) == NULL) { status = eslEMEM; goto ERROR; } } while (0)
#define ESL_REALLOC(p, newsize) do { void *shim_tmp_; \
    if ((shim_tmp_ = realloc((p), (newsize))) == NULL) { status = eslEMEM; goto ERROR; } \
    (p) = shim_tmp_; } while (0)
#define ESL_FAIL(code, errbuf, ...) do { \
    if ((errbuf) != NULL) snprintf((errbuf), eslERRBUFSIZE, __VA_ARGS__); return (code); } while (0)
#define ESL_XFAIL(code, errbuf, ...) do { status = (code); \
    if ((errbuf) != NULL) snprintf((errbuf), eslERRBUFSIZE, __VA_ARGS__); goto ERROR; } while (0)
#define ESL_EXCEPTION(code, ...) do { fprintf(stderr, __VA_ARGS__); return (code); } while (0)
#define ESL_XEXCEPTION(code, ...) do { status = (code); fprintf(stderr, __VA_ARGS__); goto ERROR; } while (0)
#define ESL_RALLOC(p, tmp, newsize) do { \
    if ((p) == NULL) { (tmp) = malloc(newsize); } else { (tmp) = realloc((p), (newsize)); } \
    if ((tmp) != NULL) (p) = (tmp); else { status = eslEMEM; goto ERROR; } } while (0)
#define ESL_DPRINTF1(x)
#define ESL_DPRINTF2(x)
#define ESL_DPRINTF3(x)
#define ESL_DASSERT1(x)
#define ESL_DASSERT2(x)
#define ESL_DASSERT3(x)

/* Alphabet: only type/K/Kp and the degeneracy table are read by the path. */
#define eslRNA 1
#define eslDNA 2
#define eslAMINO 3
typedef struct {
  int   type;
  int   K;
  int   Kp;
  char  sym[32];
  char **degen;   /* [0..Kp-1][0..K-1] flags, used by residue counting */
  int   *ndegen;
} ESL_ALPHABET;

/* Opaque easel types referenced only through pointers. */
typedef struct esl_randomness_s ESL_RANDOMNESS;
typedef struct esl_sq_s         ESL_SQ;
typedef struct esl_msa_s        ESL_MSA;
typedef struct esl_stopwatch_s  ESL_STOPWATCH;
typedef struct esl_mixdchlet_s  ESL_MIXDCHLET;
typedef struct esl_keyhash_s    ESL_KEYHASH;
typedef struct esl_getopts_s    ESL_GETOPTS;
typedef struct esl_sqfile_s     ESL_SQFILE;
typedef struct esl_dmatrix_s    ESL_DMATRIX;
typedef struct esl_ssi_s        ESL_SSI;
typedef struct esl_sq_block_s   ESL_SQ_BLOCK;
typedef struct esl_stack_s      ESL_STACK;
typedef struct esl_fileparser_s ESL_FILEPARSER;
typedef struct esl_histogram_s  ESL_HISTOGRAM;
typedef struct esl_hmm_s        ESL_HMM;
typedef struct esl_sqcache_s    ESL_SQCACHE;
typedef struct esl_options_s    ESL_OPTIONS;
#define eslSMALLX1 5e-9

/* Vector helpers (definitions in shim_easel.c). */
void   esl_vec_FSet (float  *v, int64_t n, float  x);
void   esl_vec_ISet (int    *v, int64_t n, int    x);
void   esl_vec_DSet (double *v, int64_t n, double x);
void   esl_vec_DCopy(const double *src, int64_t n, double *dest);
void   esl_vec_FCopy(const float  *src, int64_t n, float  *dest);
void   esl_vec_ICopy(const int    *src, int64_t n, int    *dest);
float  esl_vec_FSum (const float  *v, int64_t n);
double esl_vec_DSum (const double *v, int64_t n);
void   esl_vec_FNorm(float  *v, int64_t n);
void   esl_vec_DNorm(double *v, int64_t n);
void   esl_vec_FScale(float *v, int64_t n, float x);
int    esl_vec_IMax (const int *v, int64_t n);
float  esl_vec_FMax (const float *v, int64_t n);
int    esl_abc_DCount(const ESL_ALPHABET *abc, double *ct, ESL_DSQ x, double wt);
int    esl_abc_XIsCanonical(const ESL_ALPHABET *abc, ESL_DSQ x);
#define esl_abc_XIsGap(a, x) ((x) == (a)->K)

/* Sorting helper used by the hit list. */
int esl_quicksort(const void *data, int n, int (*comparison)(const void *data, int o1, int o2), int *sorted_at);
void esl_fatal(const char *format, ...);
#endif
