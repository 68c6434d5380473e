/* project-written stand-in: prototypes of the integer push-down stack that
 * CreateEmitMap (src/display.c) walks the guide tree with; the functions are
 * restated in oracle/ref_harness.c. */
#ifndef CMGB_SHIM_ESL_STACK_H
#define CMGB_SHIM_ESL_STACK_H
ESL_STACK *esl_stack_ICreate(void);
int        esl_stack_IPush(ESL_STACK *s, int x);
int        esl_stack_IPop(ESL_STACK *s, int *ret_x);
void       esl_stack_Destroy(ESL_STACK *s);
#endif
