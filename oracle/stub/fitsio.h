/*
 * Stub fitsio.h used ONLY to compile the reference's own sources into the
 * oracle library (oracle/_ref).  cfitsio is not installed; the hot path never
 * touches FITS I/O, so every routine the reference calls expands to a no-op
 * that reports success.  Only names and types are provided, no behaviour.
 */
#ifndef DEMON_ORACLE_STUB_FITSIO_H
#define DEMON_ORACLE_STUB_FITSIO_H

typedef struct fitsfile_stub fitsfile;
typedef long long LONGLONG;

#define IMAGE_HDU 0
#define BINARY_TBL 2
#define TLONG 41
#define TDOUBLE 82
#define KEY_NO_EXIST 202
#define VALUE_UNDEFINED 204
#define READONLY 0
#define READWRITE 1

#define DEMON_FITS_NOOP(...) ((void)0)
#define fits_close_file(...) DEMON_FITS_NOOP()
#define fits_create_file(...) DEMON_FITS_NOOP()
#define fits_create_img(...) DEMON_FITS_NOOP()
#define fits_create_tbl(...) DEMON_FITS_NOOP()
#define fits_file_exists(...) DEMON_FITS_NOOP()
#define fits_flush_file(...) DEMON_FITS_NOOP()
#define fits_get_num_rows(...) DEMON_FITS_NOOP()
#define fits_movabs_hdu(...) DEMON_FITS_NOOP()
#define fits_movnam_hdu(...) DEMON_FITS_NOOP()
#define fits_open_file(...) DEMON_FITS_NOOP()
#define fits_read_col_dbl(...) DEMON_FITS_NOOP()
#define fits_read_errmsg(...) DEMON_FITS_NOOP()
#define fits_read_key_dbl(...) DEMON_FITS_NOOP()
#define fits_read_key_lng(...) DEMON_FITS_NOOP()
#define fits_update_key(...) DEMON_FITS_NOOP()
#define fits_write_col_dbl(...) DEMON_FITS_NOOP()
#define fits_write_key_dbl(...) DEMON_FITS_NOOP()

#endif
