/* fitsio.h -- declarations only, so that the reference's chealpix.c compiles
 * without cfitsio.  TEST INFRASTRUCTURE ONLY: the HEALPix map readers and
 * writers built on these fail (every function returns a nonzero status); the
 * pixelisation functions of chealpix.c, which do not use them, are what the
 * checkers call. */
#ifndef OPSEC_FITSIO_STUB_H
#define OPSEC_FITSIO_STUB_H
#include <stdio.h>

typedef struct fitsfile fitsfile;

#define READONLY 0
#define READWRITE 1
#define BINARY_TBL 2
#define TSTRING 16
#define TLONG 41
#define TFLOAT 42
#define FLOAT_IMG (-32)
#define SHORT_IMG 16
#define FLEN_COMMENT 73
#define FLEN_VALUE 71
#define FLEN_KEYWORD 75
#define FLEN_CARD 81

int fits_open_file(fitsfile** f, const char* name, int mode, int* status);
int fits_create_file(fitsfile** f, const char* name, int* status);
int fits_close_file(fitsfile* f, int* status);
int fits_movabs_hdu(fitsfile* f, int hdu, int* type, int* status);
int fits_read_key_lng(fitsfile* f, const char* key, long* value, char* comment, int* status);
int fits_read_keys_lng(fitsfile* f, const char* key, int first, int n, long* values, int* found, int* status);
int fits_read_key(fitsfile* f, int type, const char* key, void* value, char* comment, int* status);
int fits_read_col(fitsfile* f, int type, int col, long long row, long long elem, long long n, void* nulval,
                  void* values, int* anynul, int* status);
int fits_create_img(fitsfile* f, int bitpix, int naxis, long* naxes, int* status);
int fits_create_tbl(fitsfile* f, int type, long long rows, int fields, char** ttype, char** tform, char** tunit,
                    const char* extname, int* status);
int fits_write_key(fitsfile* f, int type, const char* key, void* value, const char* comment, int* status);
int fits_write_comment(fitsfile* f, const char* comment, int* status);
int fits_write_date(fitsfile* f, int* status);
int fits_write_col(fitsfile* f, int type, int col, long long row, long long elem, long long n, void* values,
                   int* status);
void fits_report_error(FILE* stream, int status);

#endif
