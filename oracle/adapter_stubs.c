/* adapter_stubs.c -- TEST INFRASTRUCTURE ONLY.
 *
 * The adapter test links the reference harness (oracle/ref_harness.c) with
 * the Infernal-side adapter instead of the reference's scanner objects.  The
 * harness also names the three reference-order scanners the adapter does not
 * replace (RefCYKScan, RefIInsideScan, RefFInsideScan: the oracle forms of
 * src/cm_dpsearch.c:718, 2359, 2737); these stand-ins let the test library
 * load and report that they are not provided. */
#include "easel.h"
#include "esl_alphabet.h"
#include "hmmer.h"
#include "infernal.h"

static int not_provided(const char *name, char *errbuf)
{
  if (errbuf) snprintf(errbuf, eslERRBUFSIZE, "%s is not provided by the GPU adapter\n", name);
  return eslEINCOMPAT;
}
int RefCYKScan(CM_t *cm, char *errbuf, CM_SCAN_MX *smx, int qdbidx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff,
               CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc,
               float *ret_sc)
{ return not_provided("RefCYKScan", errbuf); }
int RefIInsideScan(CM_t *cm, char *errbuf, CM_SCAN_MX *smx, int qdbidx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff,
                   CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc,
                   float *ret_sc)
{ return not_provided("RefIInsideScan", errbuf); }
int RefFInsideScan(CM_t *cm, char *errbuf, CM_SCAN_MX *smx, int qdbidx, ESL_DSQ *dsq, int64_t i0, int64_t j0, float cutoff,
                   CM_TOPHITS *hitlist, int do_null3, float env_cutoff, int64_t *ret_envi, int64_t *ret_envj, float **ret_vsc,
                   float *ret_sc)
{ return not_provided("RefFInsideScan", errbuf); }
