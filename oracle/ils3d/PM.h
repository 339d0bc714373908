/*
 * PM.h -- project-written stand-in for SolverTest's PMlib timer macros
 * (examples/SolverTest/PM.h): PM_Start / PM_Stop discard their arguments.
 * TEST INFRASTRUCTURE ONLY (PMlib is not available here; timers do not
 * change results).
 */
#ifndef BCMG_ILS3D_PM_H
#define BCMG_ILS3D_PM_H
#define PM_Start(...) ((void)0)
#define PM_Stop(...) ((void)0)
#endif
