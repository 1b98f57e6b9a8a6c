/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiled by oracle/Makefile together with the reference's own src/doci.c,
 * read in place from the reference checkout (nothing is copied), into
 * oracle/_ref/libdoci_ref.so.  doci.c's entry points (fill_doci_data,
 * doci_matvec, ...) are exported as they are; this file only adds accessors
 * for the fields of its private struct doci_data (doci.c:9-22) that the pins
 * need: the lexical bitstring table (doci.c:472-548) and the thread count.
 */
#include "doci.c"

unsigned int *ref_to_bitstring(void *vdat) { return ((struct doci_data *)vdat)->to_bitstring; }
double *ref_viikk(void *vdat) { return ((struct doci_data *)vdat)->Viikk; }
int ref_threadnos(void *vdat) { return ((struct doci_data *)vdat)->threadnos; }
unsigned int ref_n_pairs(void *vdat) { return ((struct doci_data *)vdat)->N; }
unsigned int ref_n_orbitals(void *vdat) { return ((struct doci_data *)vdat)->L; }
