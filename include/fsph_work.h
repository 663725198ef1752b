/*
 * fsph_work.h -- the fixed algorithmic work model of the SPH step, used for
 * the roofline fractions reported by bench.py.  The same table applies to
 * both precisions: extra operations of compensated summation, of the exact
 * neighbour predicate or of recomputation are not counted as useful work.
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

/* Compulsory HBM bytes per particle and step (every field read or written
 * once per kernel, neighbour re-reads served from cache):
 *   range+keys 40, sort (key,id) 32 + permute 272, tree 48, density 72,
 *   acceleration 120, de/dt 112, kicks/drift 288, dt 80, lists 4*N_nb*5 */
#define FSPH_BYTES_PARTICLE_STEP_FP64 1100
#define FSPH_BYTES_PARTICLE_STEP_MIXED 650
/* neighbour list traffic: one int per pair written once, read by 4 passes */
#define FSPH_BYTES_PAIR_LISTS 20

#endif
