// mechanism.H — ORACLE test infrastructure: the species count of the compiled
// mechanism (PelePhysics' generated mechanism.H), set per build by
// oracle/ref_build.py (-DPC_REF_NS=1, 9 or 21).
#pragma once

#ifndef PC_REF_NS
#error "PC_REF_NS (the species count) must be defined"
#endif
#define NUM_SPECIES PC_REF_NS
