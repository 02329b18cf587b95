/*
 * Empty stand-in for Intel MKL's VSL header.  TEST INFRASTRUCTURE ONLY.
 * The reference includes it (simulation_cpu.h:11) but its only use is behind
 * "#ifdef INTEL_MKL", which the reference leaves undefined (it defines
 * INTEL_MKL1, simulation_cpu.h:18), so no declaration is needed.
 */
#ifndef HJM_ORACLE_MKL_VSL_SHIM_H
#define HJM_ORACLE_MKL_VSL_SHIM_H
#endif
