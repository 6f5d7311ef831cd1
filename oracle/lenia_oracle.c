/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * CPU oracle for the DiffusionLenia step of anima-zetta/cella-nova
 * (ml-rs/example.rs:164-303), built as liblenia_oracle.so by oracle/Makefile.
 * Exports:
 *   orc_step_f64 / orc_mass_f64 — FP64 restatement: the parity oracle
 *   orc_step_f32 / orc_mass_f32 — FP32 restatement with example.rs's own f32
 *                                 twiddle arithmetic: the timed CPU baseline
 * Parity pin: tests/golden/ holds vectors produced by the reference's own
 * PyTorch DiffusionLenia (train/diff_lenia_org.py) and tests/test_oracle.py
 * checks both builds against them.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

#define REAL double
#define SUF _f64
#define COS cos
#define SIN sin
#define EXP exp
#include "oracle_impl.h"
#undef REAL
#undef SUF
#undef COS
#undef SIN
#undef EXP

#define REAL float
#define SUF _f32
#define COS cosf
#define SIN sinf
#define EXP expf
#include "oracle_impl.h"
#undef REAL
#undef SUF
#undef COS
#undef SIN
#undef EXP
