/* ref_offpath.c -- fail-loud stand-ins for symbols that the compiled
 * reference files reference from code that is not on the scanning path
 * (alignment display, pipeline output, parse trees, Easel I/O).
 *
 * TEST INFRASTRUCTURE ONLY (part of oracle/_ref).  Kept out of
 * ref_harness.c so that these untyped stubs do not meet the reference
 * prototypes.  The scanners never reach them; they abort loudly if
 * anything does. */
#include <stdio.h>
#include <stdlib.h>
static void offpath(const char *name) { fprintf(stderr, "off-path reference function %s called\n", name); exit(1); }
#define OFFPATH(name) void name(void) { offpath(#name); }
OFFPATH(CMCountNodetype) OFFPATH(CMCountStatetype) OFFPATH(CMStateid) OFFPATH(EmitParsetree)
OFFPATH(FreeParsetree) OFFPATH(IntMaxDigits) OFFPATH(Nodetype)
OFFPATH(Parsetrees2Alignment) OFFPATH(Statetype) OFFPATH(cm_alidisplay_Backconvert) OFFPATH(cm_alidisplay_Destroy)
OFFPATH(cm_alidisplay_Dump) OFFPATH(cm_alidisplay_Is3PTrunc) OFFPATH(cm_alidisplay_Is5PTrunc)
OFFPATH(cm_alidisplay_Print) OFFPATH(cm_alidisplay_TruncString) OFFPATH(cm_pli_TargetIncludable)
OFFPATH(cm_pli_TargetReportable) OFFPATH(esl_DCompare_old) OFFPATH(esl_getcwd) OFFPATH(esl_keyhash_Get)
OFFPATH(esl_keyhash_GetNumber) OFFPATH(esl_msa_Destroy) OFFPATH(esl_opt_SpoofCmdline)
OFFPATH(esl_randomness_CreateTimeseeded) OFFPATH(esl_randomness_Destroy) OFFPATH(esl_sq_Destroy)
OFFPATH(AllocCP9Bands) OFFPATH(CMLogoddsify) OFFPATH(CP9Logoddsify) OFFPATH(CreateCP9Matrix)
OFFPATH(DegeneratePairScore) OFFPATH(SubCMLogoddsify) OFFPATH(build_cp9_hmm) OFFPATH(cm_Validate)
OFFPATH(cm_cp9_to_p7) OFFPATH(cm_nonconfigured_Verify) OFFPATH(cp9_Clone) OFFPATH(esl_abc_FAvgScore)
OFFPATH(esl_strcat) OFFPATH(esl_strchop) OFFPATH(esl_strdup) OFFPATH(esl_vec_FArgMax)
OFFPATH(sub_build_cp9_hmm_from_mother)
