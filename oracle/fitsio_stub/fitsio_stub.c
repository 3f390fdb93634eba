/* fitsio_stub.c -- definitions for fitsio.h in this directory.  TEST
 * INFRASTRUCTURE ONLY: every call fails with status 104 (file not found). */
#include "fitsio.h"

#define FAIL { if (status) *status = 104; return 104; }
int fits_open_file(fitsfile** f, const char* name, int mode, int* status) { (void)f; (void)name; (void)mode; FAIL }
int fits_create_file(fitsfile** f, const char* name, int* status) { (void)f; (void)name; FAIL }
int fits_close_file(fitsfile* f, int* status) { (void)f; FAIL }
int fits_movabs_hdu(fitsfile* f, int hdu, int* type, int* status) { (void)f; (void)hdu; (void)type; FAIL }
int fits_read_key_lng(fitsfile* f, const char* key, long* value, char* comment, int* status) {
    (void)f; (void)key; (void)value; (void)comment; FAIL }
int fits_read_keys_lng(fitsfile* f, const char* key, int first, int n, long* values, int* found, int* status) {
    (void)f; (void)key; (void)first; (void)n; (void)values; (void)found; FAIL }
int fits_read_key(fitsfile* f, int type, const char* key, void* value, char* comment, int* status) {
    (void)f; (void)type; (void)key; (void)value; (void)comment; FAIL }
int fits_read_col(fitsfile* f, int type, int col, long long row, long long elem, long long n, void* nulval,
                  void* values, int* anynul, int* status) {
    (void)f; (void)type; (void)col; (void)row; (void)elem; (void)n; (void)nulval; (void)values; (void)anynul; FAIL }
int fits_create_img(fitsfile* f, int bitpix, int naxis, long* naxes, int* status) {
    (void)f; (void)bitpix; (void)naxis; (void)naxes; FAIL }
int fits_create_tbl(fitsfile* f, int type, long long rows, int fields, char** ttype, char** tform, char** tunit,
                    const char* extname, int* status) {
    (void)f; (void)type; (void)rows; (void)fields; (void)ttype; (void)tform; (void)tunit; (void)extname; FAIL }
int fits_write_key(fitsfile* f, int type, const char* key, void* value, const char* comment, int* status) {
    (void)f; (void)type; (void)key; (void)value; (void)comment; FAIL }
int fits_write_comment(fitsfile* f, const char* comment, int* status) { (void)f; (void)comment; FAIL }
int fits_write_date(fitsfile* f, int* status) { (void)f; FAIL }
int fits_write_col(fitsfile* f, int type, int col, long long row, long long elem, long long n, void* values,
                   int* status) { (void)f; (void)type; (void)col; (void)row; (void)elem; (void)n; (void)values; FAIL }
void fits_report_error(FILE* stream, int status) { (void)stream; (void)status; }
