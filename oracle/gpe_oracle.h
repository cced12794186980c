/*
 * gpe_oracle.h -- FP64 CPU restatement of the reference's per-step kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA path of libgpe is
 * compared against (and the timed CPU baseline of bench.py).  Nothing in the
 * library links or calls it.
 *
 * Buffers use the reference file layout: (Z+2)(Y+2)(X+2) cells, x fastest, a
 * one-cell zero halo on every side; a psi cell holds V nodes x C components x
 * (re, im) doubles, a q cell E edges x C components x (re, im).
 */
#ifndef GPE_ORACLE_H
#define GPE_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/gpe.h"

#ifdef __cplusplus
extern "C" {
#endif

/* step modes */
enum {
    ORC_LEAPFROG = 0,   /* next += 2 dt (-i H prev) */
    ORC_EULER = 1,      /* next  = prev + dt (-i H prev) */
    ORC_ITP = 2         /* hpsi = H prev; next = prev - dt H prev */
};

/* q modes */
enum {
    ORC_Q_HYPER = 0,      /* next_q += i 2 (dt/sigma) (prev_q + d0 psi)       */
    ORC_Q_PARA = 1,       /* next_q  = d0 psi                                  */
    ORC_Q_EULER_HYPER = 2, /* next_q  = prev_q + i (dt/sigma) (prev_q + d0 psi) */
    ORC_Q_ITP = 3          /* next_q  = prev_q - (dt/sigma) (prev_q - d0 psi)  */
};

/* Parabolic step for C = 1, 3, 5 (scalar GPUGrossPitaevskii_BCC.cu:327-347;
 * spin-1 Spin1GpeBCC.cu:554-917; spin-2 Spin2GpeBCC.cu:561-990).
 * `threads` > 1 splits the z range over OpenMP threads (0 = all). */
int orc_parabolic_step(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* B,
                       double t, int mode, double* next, const double* prev, double* hpsi,
                       int threads);

/* Hyperbolic / q-based psi update for C = 1, 3, 5 (update_psi and forwardEuler:
 * RelativisticGpeBCC.cu:212-255, RelativisticSpin1Gpe/common_kernels.h:95-255,
 * RelativisticSpin2Gpe.cu:859-969, 1022-1132).  hyperb selects the -c_K scaling.
 * mode ORC_ITP with hyperb = 0 is the imaginary-time itp_psi (B = 0; hpsi, when
 * not NULL, receives H prev: RelativisticSpin2Gpe.cu:706-807 and get_Hpsi :602-704,
 * RelativisticSpin1Gpe/common_kernels.h:17-94). */
int orc_q_psi_step(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* B,
                   double t, int mode, int hyperb, double* next, const double* prev,
                   const double* q, double* hpsi, int threads);

/* Dual-edge update (update_q / forwardEuler_q / update_q_para / itp_q:
 * RelativisticSpin2Gpe.cu:558-599, 808-857, 971-1020; RelativisticSpin1Gpe/hyper_kernels.h:4-40,
 * 80-116, para_kernels.h:4-31; RelativisticGpeBCC.cu:154-210).  next_q may equal
 * prev_q (each edge reads only its own prev_q). */
int orc_q_step(const gpe_lattice_desc* lat, const gpe_params* p, int qmode,
               double* next_q, const double* prev_q, const double* psi, int threads);

/* Per-node output fields (GPE_FIELD_*; gpe_node_fields), interior nodes in the
 * reference's order idx = V (z X Y + y X + x) + l. */
int orc_node_fields(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* B, double t, int kind,
                    const double* psi, double* out);

/* Real/imaginary split scalar scheme (RelativisticGpeC15/GPUGrossPitaevskii_C15.cu:
 * 90-155, 469, 477-482) on complex-pair buffers psi = R + iI, q = q_R + i q_I, in
 * place.  part 0: I and q_I from R and q_R; part 1: R and q_R from I and q_I; part 2:
 * the start q_R += c (q_R + d0 R), c = (dt/sigma) / (dt - dt/sigma). */
int orc_split_step(const gpe_lattice_desc* lat, const gpe_params* p, int part, double* psi, double* q,
                   int threads);

/* Renormalise psi to unit norm, sum |psi|^2 dv = 1 (density + integrate + normalize,
 * Spin1GpeBCC.cu:191-211, 328-348, 412-434).  Returns the norm before scaling. */
double orc_normalize(const gpe_lattice_desc* lat, const gpe_params* p, double* psi);

/* FP64 observables (see gpe_observables in gpe.h for the definitions). */
int orc_observe(const gpe_lattice_desc* lat, const gpe_params* p, const gpe_fields* B,
                double t, const double* psi, gpe_observables* out);

/* Field ramp (getSignal + scaling, Spin1GpeBCC/AliceRingRamps.h:74-141). */
void orc_ramp_eval(const gpe_ramp* r, double tau, gpe_fields* out);

/* GPBlocks CPU stepper restated (GrossPitaevskii/GPBlocks.cpp:451-609) on its own
 * flat layout: bsize=V, bxsize=(X+1)V, bxysize=(Y+1)bxsize, ii0=bxysize+bxsize+V,
 * vsize = ii0 + (Z+1)bxysize complex values.  lapind holds V*deg flat offsets,
 * pot and g are already multiplied by the time step, as in the reference.
 * Runs `steps` double steps (odd <- even, then even <- odd). */
void orc_gpblocks_run(int X, int Y, int Z, int V, int deg, const int64_t* lapind,
                      double lapfac, double lapfac0, double g, const double* pot,
                      double* even, double* odd, int steps);

/* sum |psi|^2 * volume over flat indices [ii0, vsize) and <psi0|psi> * volume
 * (GPBlocks.cpp:531-538).  out[0] = normsq, out[1] = normsq - |error|. */
void orc_gpblocks_norm(size_t ii0, size_t vsize, const double* psi0, const double* even,
                       double volume, double out[2]);

#ifdef __cplusplus
}
#endif
#endif
