// Status codes and counters shared by the CUDA kernels and the C-ABI.
#pragma once

// Return codes of the C-ABI entry points.
#define PG_OK 0
#define PG_EARG -1          // invalid sizes or null pointers
#define PG_EWORKSPACE -2    // workspace smaller than the size query returned
#define PG_ECUDA -3         // a CUDA launch failed (cudaGetLastError)
#define PG_ETOOBIG -4       // request exceeds a fixed capacity of the entry point

// Bits of the device status word written by the weight kernel.  Each bit
// marks a condition where the reference stops the process (or has undefined
// behaviour); the affected (tetrahedron, band pair) contributes zero.
#define PG_ERR_NNOD (1u << 0)       // convw1t_par: nnod > 8 (for_tetrahedra3.f90:121-123)
#define PG_ERR_SORTEQ (1u << 1)     // sorteq default case (for_tetrahedra2.f90:1777-1781)
#define PG_ERR_SORTNODES (1u << 2)  // sortnodes stops (for_tetrahedra2.f90:2767-2769 and siblings)
#define PG_ERR_RELNODES (1u << 3)   // relnodes ntype out of range (for_tetrahedra2.f90:2241-2244)
#define PG_ERR_EQUIV (1u << 4)      // stweight_imag_par bad equiv_flag (for_tetrahedra3.f90:687-690)
#define PG_ERR_UNDEFINED (1u << 5)  // reference reads uninitialised data / writes through index 0
#define PG_ERR_NONFINITE (1u << 6)  // a non-finite weight was produced
#define PG_ERR_TIMEOUT (1u << 7)    // a bounded wait inside a pipelined kernel expired

// Counters (unsigned long long) accumulated by the weight kernel; the same
// layout as the oracle's statistics.
#define PG_CNT_CALLS 0             // convw1t_par calls (non-skipped tetrahedron × band pair)
#define PG_CNT_NNOD0 1             // 1..9: polyhedron node count 0..8
#define PG_CNT_EQ4 10              // 10..14: sorteq grouping 4, 6, 8, 10, 16
#define PG_CNT_TAYLOR 15           // (sub-tetrahedron, ω) evaluated by the Taylor series
#define PG_CNT_EXACT 16            // (sub-tetrahedron, ω) evaluated in closed form
#define PG_CNT_ZERO_VOL 17         // sub-tetrahedra below the volume tolerance
#define PG_CNT_BIGW_WARN 18        // |w| > 1e4 at ω ≥ 1e-6 (reference prints a warning)
#define PG_CNT_BIGW_ZEROED 19      // |w| > 1e4 at ω < 1e-6 (reference zeroes it)
#define PG_NCOUNTERS 20

// Size of the device array used by pg_bz_calcqdepw_par2_noalloc (256 MiB).
#define PG_NOALLOC_SCRATCH_BYTES (256ull << 20)
