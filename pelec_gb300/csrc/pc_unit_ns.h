// pc_unit_ns.h — splitting a translation unit's species-count instantiations
// over several compilations.  pelec_gb300/build.py compiles the units with
// the heaviest kernels (the flux pass at the other tile shapes, the adjoint,
// the tangent) once per species count, with -DPC_UNIT_NS=<count>; each
// compilation explicitly instantiates its count's functions and declares the
// others extern, and the one-species compilation holds the dispatcher.
// Without PC_UNIT_NS a unit instantiates every count.
#pragma once

#ifdef PC_UNIT_NS
#define PC_UNIT_HAS(ns) (PC_UNIT_NS == (ns))
#else
#define PC_UNIT_HAS(ns) 1
#endif

#define PC_UNIT_ONE(INST, ns) PC_UNIT_ONE_##ns(INST)
// INST(ns) expands to an explicit instantiation definition; prefixed with
// `extern` it is a declaration.
#if PC_UNIT_HAS(1)
#define PC_UNIT_ONE_1(INST) INST(1)
#else
#define PC_UNIT_ONE_1(INST) extern INST(1)
#endif
#if PC_UNIT_HAS(9)
#define PC_UNIT_ONE_9(INST) INST(9)
#else
#define PC_UNIT_ONE_9(INST) extern INST(9)
#endif
#if PC_UNIT_HAS(21)
#define PC_UNIT_ONE_21(INST) INST(21)
#else
#define PC_UNIT_ONE_21(INST) extern INST(21)
#endif
#define PC_UNIT_INSTANTIATE(INST) \
  PC_UNIT_ONE(INST, 1)            \
  PC_UNIT_ONE(INST, 9)            \
  PC_UNIT_ONE(INST, 21)
