/* project-written stand-in: the two fields of Easel's getopts object that
 * display.c reads (GetCommand); nothing on the scanning path uses them. */
#ifndef CMGB_SHIM_ESL_GETOPTS_H
#define CMGB_SHIM_ESL_GETOPTS_H
struct esl_getopts_s { int argc; char **argv; };
#endif
