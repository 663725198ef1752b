/*
 * fsph_work.h -- the fixed algorithmic work model of the SPH step.  The
 * roofline fractions bench.py reports are computed from these constants
 * (bench.py parses this file), and nothing else: the same table serves both
 * precisions, because extra operations of compensated or float-float
 * arithmetic, of the exact neighbour predicate, of recomputation, or bytes
 * an implementation moves beyond the compulsory ones are not useful work.
 * What an implementation really moves is reported beside it as `traffic`
 * (ncu dram bytes).
 *
 * Flops per neighbour pair count +, -, *, /, sqrt as one each, as the
 * reference writes the pair terms (include/physics/default_physics.h,
 * kernels.h, viscosity.h); Wendland C6 in 3D.
 */
#ifndef FSPH_WORK_H
#define FSPH_WORK_H

#define FSPH_FLOPS_PAIR_DENSITY 31   /* r, W(r, h_ab), rho += m W            */
#define FSPH_FLOPS_PAIR_VSIG 27      /* n_ab, v_ab . n_ab, max(...)          */
#define FSPH_FLOPS_PAIR_ACCEL 82     /* mu, Pi, grad W, P/rho^2 terms         */
#define FSPH_FLOPS_PAIR_DUDT 84
#define FSPH_FLOPS_PAIR_DEDT 96
#define FSPH_FLOPS_PAIR_P2P 22       /* gravity particle-particle            */
#define FSPH_FLOPS_PAIR_M2P_QUAD 62  /* monopole 22 + quadrupole 40          */

/* Compulsory HBM bytes per particle and step, by phase: FP64 SoA in 3D,
 * every field read or written once per kernel, neighbour re-reads served
 * from cache.  The state is FP64 in both precision modes. */
#define FSPH_BYTES_RANGE_KEYS 40     /* x, y, z, h read; key written          */
#define FSPH_BYTES_SORT 304          /* (key, id) 2 x 16 + permute 2 x 17 x 8 */
#define FSPH_BYTES_TREE 48
#define FSPH_BYTES_NEIGHBORS 40      /* x, y, z, h read; count written       */
#define FSPH_BYTES_DENSITY 72        /* 40 in + 32 out                       */
#define FSPH_BYTES_ACCEL 120         /* 96 in + 24 out                       */
#define FSPH_BYTES_DEDT 112          /* 104 in + 8 out                       */
#define FSPH_BYTES_RECOMPUTE_P 40
#define FSPH_BYTES_INTEGRATE 288     /* kicks, drift, v_half: 3 x 96         */
#define FSPH_BYTES_DT 80
/* the neighbour list: one int per pair, written by the walk and read by
 * each pair pass */
#define FSPH_BYTES_PAIR_LIST 4

/* totals per particle-step (hydro, thermokinetic) */
#define FSPH_BYTES_PARTICLE_STEP_FP64 1104
/* ...and if non-position fields were stored in FP32 (not done here: the
 * leapfrog state stays FP64) */
#define FSPH_BYTES_PARTICLE_STEP_MIXED 650
/* list traffic per pair and step: written once, read by 4 passes */
#define FSPH_BYTES_PAIR_LISTS 20

#endif
