/* MSVC <zmmintrin.h> stand-in for the reference build on Linux/x86 (oracle recipe
 * only). Besides pulling in the AVX-512 intrinsics it maps two MSVC-only spellings
 * the reference's AVX-512 utilities use onto their GCC equivalents:
 *  - _mm512_permutevar_epi32(idx, a) is the KNC name of _mm512_permutexvar_epi32;
 *  - MSVC keeps the low 8 bits of an over-wide _mm512_shuffle_ps immediate, GCC
 *    rejects it, so the immediate is masked the way MSVC treats it. */
#pragma once
#include <immintrin.h>
#define _mm512_permutevar_epi32(idx, a) _mm512_permutexvar_epi32((idx), (a))
#ifdef __OPTIMIZE__
#define _mm512_shuffle_ps(a, b, imm) (_mm512_shuffle_ps)((a), (b), (imm) & 0xFF)
#endif
/* The reference's debug print helpers name two extract intrinsics GCC lacks; they
 * are never called on the sort path, so they only need to compile. */
#define _mm256_extract_pd(a, i) 0.0
#define _mm512_extractf64x4_pd(a, i) _mm256_setzero_pd()
