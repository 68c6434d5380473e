/* Minimal stand-in for the HMMER header, written for this project: the
 * scanner path only passes these types around as opaque pointers. */
#ifndef INFGB_SHIM_HMMER_H
#define INFGB_SHIM_HMMER_H
typedef struct p7_profile_s    P7_PROFILE;
typedef struct p7_hmm_s        P7_HMM;
typedef struct p7_gmx_s        P7_GMX;
typedef struct p7_oprofile_s   P7_OPROFILE;
typedef struct p7_omx_s        P7_OMX;
typedef struct p7_bg_s         P7_BG;
typedef struct p7_trace_s      P7_TRACE;
typedef struct p7_scoredata_s  P7_SCOREDATA;
typedef struct p7_domaindef_s  P7_DOMAINDEF;
typedef struct p7_alidisplay_s P7_ALIDISPLAY;
typedef struct p7_hmmfile_s    P7_HMMFILE;
typedef struct p7_pipeline_s   P7_PIPELINE;
typedef struct p7_tophits_s    P7_TOPHITS;
typedef struct p7_hit_s        P7_HIT;
typedef struct p7_filtermx_s   P7_FILTERMX;
typedef struct p7_checkptmx_s  P7_CHECKPTMX;
#define p7_NEVPARAM 6
#define p7_NCUTOFFS 6
#define p7_MAXABET  20
#endif
