/**
 * FitsLite.h -- the FITS subset the reference's output files use, without
 * cfitsio.
 *
 * The reference writes (driver.cpp:360-366, Cloud.cpp:190-271, each
 * Force::writeForce):
 *  - a primary HDU with no data (16-bit, NAXIS = 0) whose header carries
 *    FORCES (the ForceFlag bitmask) and each force's parameters
 *    (confineConst, shieldingConstant, ...);
 *  - a binary table CLOUD: one row per particle, columns MASS [kg] and
 *    CHARGE [C] (TFORM 'D');
 *  - a binary table TIME_STEP: one row per output time, columns TIME [s]
 *    ('D') and X_POSITION, Y_POSITION [m], X_VELOCITY, Y_VELOCITY [m/s]
 *    ('<n>D'), rows appended as the run goes, each flushed to disk.
 * This file writes and reads exactly that: tables whose columns are all
 * FP64 vectors, appended row by row at the end of the file, and header keys
 * with long or double values (names over 8 characters use the HIERARCH
 * convention, as cfitsio writes them).  Status codes follow cfitsio's
 * numbering for the cases that occur.
 */
#ifndef DEMON_GB300_FITSLITE_H
#define DEMON_GB300_FITSLITE_H

#include <string>
#include <vector>

/// An open FITS file (the reference's functions take `fitsfile *`; this is
/// this library's own type, not cfitsio's).
struct fitsfile;

namespace demon_gb300 {
namespace fits {

enum Status {
    OK = 0,
    FILE_NOT_OPENED = 104,
    FILE_NOT_CREATED = 105,
    WRITE_ERROR = 106,
    READ_ERROR = 108,
    BAD_HEADER = 207,   // malformed header card or structure
    KEY_NO_EXIST = 202,
    BAD_HDU_NUM = 301,  // no HDU of that name
    NOT_BTABLE = 227,   // table structure this subset does not handle
    BAD_ROW_NUM = 307,
    STATE_ERROR = 115   // call not valid in the file's current state
};

struct Column {
    std::string name;  //!< TTYPE
    long repeat;       //!< TFORM = '<repeat>D'
    std::string unit;  //!< TUNIT
};

/// New file (truncating `path`) with an empty primary HDU.  Header keys may
/// be added until the first table is created.
fitsfile *create(const std::string &path, int &status);
/// Existing file; `readwrite` allows appending rows to its last table.
fitsfile *open(const std::string &path, bool readwrite, int &status);
void close(fitsfile *f, int &status);
/// Writes everything buffered to disk (stdio flush).
void flush(fitsfile *f, int &status);

/// Primary-header keys: add, or replace the value of an existing key.
void write_key_long(fitsfile *f, const std::string &name, long value, const std::string &comment,
                    int &status);
void write_key_dbl(fitsfile *f, const std::string &name, double value, const std::string &comment,
                   int &status);
/// Reads a primary-header key (KEY_NO_EXIST if absent).
long read_key_long(fitsfile *f, const std::string &name, int &status);
double read_key_dbl(fitsfile *f, const std::string &name, int &status);

/// Appends a binary table with FP64 columns and no rows.
void create_table(fitsfile *f, const std::string &extname, const std::vector<Column> &cols, int &status);
/// Appends `nrows` rows to the table `extname`, which must be the file's
/// last HDU.  cols[c] holds nrows * repeat_c values, row after row.
void append_rows(fitsfile *f, const std::string &extname, long nrows, const std::vector<const double *> &cols,
                 int &status);
long num_rows(fitsfile *f, const std::string &extname, int &status);
/// Column `col` (0-based) of row `row` (0-based): `repeat` values.
std::vector<double> read_cell(fitsfile *f, const std::string &extname, int col, long row, int &status);
/// Column `col` of every row, concatenated.
std::vector<double> read_column(fitsfile *f, const std::string &extname, int col, int &status);

}  // namespace fits
}  // namespace demon_gb300

#endif  // DEMON_GB300_FITSLITE_H
