/* Minimal stand-in for the Madagascar RSF C API (librsf / libsu), written for
 * this project so that the reference's CPU programs compile unchanged from
 * their own sources.  It implements only what those programs call:
 * command-line parameters (key=value), RSF headers with a separate binary
 * file (data_format=native_float, esize=4), axes, allocation helpers and the
 * pt2d/pt3d point types of libsu.
 *
 * This is test infrastructure (the oracle's checker), not product code. */
#ifndef AWE_RSF_SHIM_H
#define AWE_RSF_SHIM_H

#include <stdbool.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include <unistd.h>
#include <sys/types.h>
#ifndef __cplusplus
#include <complex.h>
typedef float _Complex sf_complex;
#endif

/* sample types (the subset the programs use) */
typedef enum { SF_UCHAR, SF_CHAR, SF_INT, SF_FLOAT, SF_COMPLEX } sf_datatype;

#define SF_PI (3.14159265358979323846264338328)
#define SF_MAX(a, b) ((a) < (b) ? (b) : (a))
#define SF_MIN(a, b) ((a) < (b) ? (a) : (b))
#define SF_ABS(a) ((a) >= 0 ? (a) : (-(a)))

typedef struct sf_File *sf_file;
typedef struct sf_Axis *sf_axis;

typedef struct {
    float x, z, v;
} pt2d;
typedef struct {
    float x, y, z, v;
} pt3d;
typedef struct {
    float dx, dy, dz;
} vc3d;

#ifdef __cplusplus
extern "C" {
#endif

void sf_init(int argc, char **argv);
bool sf_getbool(const char *key, bool *par);
bool sf_getint(const char *key, int *par);
bool sf_getfloat(const char *key, float *par);
char *sf_getstring(const char *key);

sf_file sf_input(const char *tag);
sf_file sf_output(const char *tag);

sf_axis sf_iaxa(sf_file f, int i);
void sf_oaxa(sf_file f, sf_axis a, int i);
sf_axis sf_maxa(int n, float o, float d);
void sf_raxa(sf_axis a);
int sf_n(sf_axis a);
float sf_o(sf_axis a);
float sf_d(sf_axis a);
void sf_setn(sf_axis a, int n);
void sf_seto(sf_axis a, float o);
void sf_setd(sf_axis a, float d);
void sf_setlabel(sf_axis a, const char *label);
void sf_setunit(sf_axis a, const char *unit);

void sf_floatread(float *arr, size_t n, sf_file f);
void sf_floatwrite(float *arr, size_t n, sf_file f);
void sf_settype(sf_file f, sf_datatype t);
sf_datatype sf_gettype(sf_file f);
void sf_fileclose(sf_file f);
bool *sf_boolalloc(size_t n);
off_t *sf_largeintalloc(size_t n);
#ifndef __cplusplus
sf_complex *sf_complexalloc(size_t n);
void sf_complexread(sf_complex *arr, size_t n, sf_file f);
void sf_complexwrite(sf_complex *arr, size_t n, sf_file f);
#endif
void sf_seek(sf_file f, off_t offset, int whence);

void *sf_alloc(size_t n, size_t size);
float *sf_floatalloc(size_t n);
float **sf_floatalloc2(size_t n1, size_t n2);
float ***sf_floatalloc3(size_t n1, size_t n2, size_t n3);
int *sf_intalloc(size_t n);
int **sf_intalloc2(size_t n1, size_t n2);

void sf_warning(const char *format, ...);
void sf_error(const char *format, ...);

/* libsu point helpers */
void pt2dread1(sf_file F, pt2d *v, size_t n, int k);
void pt3dread1(sf_file F, pt3d *v, size_t n, int k);
pt2d *pt2dalloc1(size_t n);
pt3d *pt3dalloc1(size_t n);
void printpt2d(pt2d P);
void printpt3d(pt3d P);
void ints8r(int nxin, float dxin, float fxin, float yin[], float yinl, float yinr, int nxout, float xout[], float yout[]);

#ifdef __cplusplus
}
#endif

#endif
