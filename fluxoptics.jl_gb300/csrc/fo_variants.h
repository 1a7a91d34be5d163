// Launch-shape variants of the row and column passes, per transform length N.
// Row: X(index, E, LANES) with E elements per thread and LANES rows per CTA.
// Column: X(index, E, W, P) with W columns per CTA; P = 1: one column per thread
// (column-fastest mapping), P = 2: paired columns, P = 0: lane-major mapping
// with a named barrier per column, P = 4: tiles staged by TMA (cp.async.bulk.tensor),
// P = 6: TMA staging with the FFT twiddles held in registers for the CTA's lifetime.  The autotuner picks among them at plan creation;
// index 0 is the default.
#pragma once

#define FO_ROW_VARIANTS_16(X) X(0, 4, 32)
#define FO_ROW_VARIANTS_32(X) X(0, 4, 16)
#define FO_ROW_VARIANTS_64(X) X(0, 8, 16)
#define FO_ROW_VARIANTS_128(X) X(0, 8, 16)
#define FO_ROW_VARIANTS_256(X) X(0, 16, 8) X(1, 8, 8)
#define FO_ROW_VARIANTS_512(X) X(0, 8, 4) X(1, 16, 4) X(2, 8, 2)
#define FO_ROW_VARIANTS_1024(X) X(0, 8, 2) X(1, 16, 2) X(2, 16, 4) X(3, 8, 1)
#define FO_ROW_VARIANTS_2048(X) X(0, 8, 1) X(1, 16, 2) X(2, 8, 2) X(3, 16, 1)
#define FO_ROW_VARIANTS_4096(X) X(0, 16, 1) X(1, 8, 1)

#define FO_COL_VARIANTS_16(X) X(0, 4, 32, 1)
#define FO_COL_VARIANTS_32(X) X(0, 4, 16, 1)
#define FO_COL_VARIANTS_64(X) X(0, 8, 16, 1)
#define FO_COL_VARIANTS_128(X) X(0, 8, 16, 1) X(1, 8, 16, 2)
#define FO_COL_VARIANTS_256(X) X(0, 16, 16, 1) X(1, 8, 8, 1) X(2, 8, 8, 2)
#define FO_COL_VARIANTS_512(X) X(0, 8, 8, 1) X(1, 16, 8, 1) X(2, 8, 4, 1) X(3, 8, 4, 2) X(4, 16, 4, 4) X(5, 8, 4, 4) X(6, 16, 2, 6) X(7, 16, 4, 6) X(8, 16, 8, 6)
#define FO_COL_VARIANTS_1024(X) X(0, 16, 4, 1) X(1, 8, 4, 1) X(2, 16, 8, 1) X(3, 8, 4, 2) X(4, 16, 4, 0) X(5, 16, 4, 4) X(6, 16, 2, 4) X(7, 16, 2, 6) X(8, 16, 4, 6) X(9, 16, 8, 6)
#define FO_COL_VARIANTS_2048(X) X(0, 16, 4, 1) X(1, 8, 4, 1) X(2, 16, 2, 1) X(3, 8, 4, 2) X(4, 16, 4, 0) X(5, 16, 4, 4) X(6, 16, 2, 4) X(7, 16, 2, 6) X(8, 16, 4, 6)
#define FO_COL_VARIANTS_4096(X) X(0, 16, 2, 1) X(1, 8, 2, 1) X(2, 16, 4, 1) X(3, 16, 2, 0) X(4, 16, 2, 4) X(5, 16, 2, 6)

#define FO_FOR_EACH_N(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)
