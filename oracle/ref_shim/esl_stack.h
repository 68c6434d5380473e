/* project-written stand-in: prototypes of Easel's push-down stacks that
 * CreateEmitMap (src/display.c, integers) and BandCalculationEngine
 * (src/cm_qdband.c, pointers) use; the functions are restated in
 * oracle/ref_harness.c. */
#ifndef CMGB_SHIM_ESL_STACK_H
#define CMGB_SHIM_ESL_STACK_H
ESL_STACK *esl_stack_ICreate(void);
int        esl_stack_IPush(ESL_STACK *s, int x);
int        esl_stack_IPop(ESL_STACK *s, int *ret_x);
void       esl_stack_Destroy(ESL_STACK *s);
ESL_STACK *esl_stack_PCreate(void);
int        esl_stack_PPush(ESL_STACK *s, void *p);
int        esl_stack_PPop(ESL_STACK *s, void **ret_p);
#endif
