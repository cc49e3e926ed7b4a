/* RSF (Madagascar) file I/O and key=value parameters for the drop-in
 * programs.  Covers what sfAWEFD*gpu and the point-cloud tools read and
 * write: float32 samples (data_format=native_float) or complex64
 * (native_complex, read and written as pairs of floats), up to 9 axes,
 * headers with a separate binary (in="path") or with the samples inline
 * after the 0x0c 0x0c 0x04 mark.  The tags "in" and "out" are standard
 * input and output; any other tag names a file on the command line
 * (tag=path), and rsf_input_path opens a header by its path. */
#ifndef AWE_RSFIO_H
#define AWE_RSFIO_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rsf_file rsf_file;

void rsf_init(int argc, char **argv);
int rsf_get_int(const char *key, int *v);
int rsf_get_float(const char *key, float *v);
int rsf_get_bool(const char *key, int *v); /* y/n, 1/0, true/false */
const char *rsf_get_string(const char *key);

rsf_file *rsf_input(const char *tag);  /* NULL + message on failure */
rsf_file *rsf_input_path(const char *path);
int rsf_is_complex(const rsf_file *f);
void rsf_set_complex(rsf_file *f, int on); /* outputs: native_complex, esize=8 */
rsf_file *rsf_output(const char *tag);
const char *rsf_error(void);

int rsf_n(const rsf_file *f, int axis); /* axis 1..9; 1 if absent */
float rsf_o(const rsf_file *f, int axis);
float rsf_d(const rsf_file *f, int axis);
size_t rsf_size(const rsf_file *f); /* product of all n */
void rsf_set_axis(rsf_file *f, int axis, int n, float o, float d, const char *label);

/* read/write float32 values in file order (a complex sample is two);
 * return values moved */
size_t rsf_read(rsf_file *f, float *buf, size_t n);
size_t rsf_write(rsf_file *f, const float *buf, size_t n);
int rsf_close(rsf_file *f); /* flushes and writes the final header of outputs */

#ifdef __cplusplus
}
#endif
#endif
