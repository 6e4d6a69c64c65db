/* Stand-in for CWP/SU su.h: the reference uses only PI, TRUE and FALSE from it. */
#ifndef OSE_REFEMU_SU_H
#define OSE_REFEMU_SU_H
#define PI (3.141592653589793)
#define TRUE (1)
#define FALSE (0)
#endif
