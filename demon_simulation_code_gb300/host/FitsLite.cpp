/**
 * FitsLite.cpp -- FITS primary header + FP64 binary tables, written and read
 * with stdio.  FITS layout: 2880-byte blocks; headers are 80-character ASCII
 * cards ending with END; table data are big-endian rows of NAXIS1 bytes,
 * padded with zeros to a whole block.
 */
#include "FitsLite.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>

namespace {
constexpr long kBlock = 2880;
constexpr int kCard = 80;

struct Hdu {
    std::string extname;      // "" for the primary HDU
    long header_off = 0;      // file offset of the first card
    long header_len = 0;      // bytes, a multiple of kBlock
    long data_off = 0;        // file offset of the data
    long naxis1 = 0, naxis2 = 0;
    long naxis2_card = -1;    // file offset of the NAXIS2 card
    std::vector<demon_gb300::fits::Column> cols;
    std::map<std::string, std::string> keys;  // name (upper case) -> raw value text
};

std::string upper(std::string s) {
    for (char &c : s) c = (char)((c >= 'a' && c <= 'z') ? c - 32 : c);
    return s;
}

long round_block(long n) { return (n + kBlock - 1) / kBlock * kBlock; }

}  // namespace

struct fitsfile {
    FILE *fp = nullptr;
    bool writable = false;
    bool primary_pending = false;           // new file: primary header not on disk yet
    std::vector<std::string> primary_cards;  // pending primary cards (without END)
    std::vector<Hdu> hdus;                   // hdus[0] = primary
};

namespace demon_gb300 {
namespace fits {

namespace {

std::string pad_card(const std::string &s) {
    std::string c = s.substr(0, kCard);
    c.resize(kCard, ' ');
    return c;
}

std::string fmt_dbl(double v) {
    char b[40];
    std::snprintf(b, sizeof b, "%.16E", v);
    return b;
}

// "NAME    = " + value right-justified to column 30 + " / comment"; names
// over 8 characters (or with lower case) as HIERARCH cards.
std::string value_card(const std::string &name, const std::string &value, const std::string &comment) {
    std::string c;
    if (name.size() <= 8 && upper(name) == name) {
        c = name;
        c.resize(8, ' ');
        c += "= ";
        std::string v = value;
        if (v.size() < 20) v = std::string(20 - v.size(), ' ') + v;
        c += v;
    } else {
        c = "HIERARCH " + name + " = " + value;
    }
    if (!comment.empty() && c.size() + 3 < (size_t)kCard) c += " / " + comment;
    return pad_card(c);
}

std::string string_card(const std::string &name, const std::string &value) {
    std::string v = value;
    if (v.size() < 8) v.resize(8, ' ');
    std::string c = name;
    c.resize(8, ' ');
    return pad_card(c + "= '" + v + "'");
}

// Parses one card into (name, raw value); false for cards without a value.
bool parse_card(const char *card, std::string &name, std::string &value) {
    std::string c(card, kCard);
    size_t eq;
    if (c.compare(0, 9, "HIERARCH ") == 0) {
        eq = c.find('=');
        if (eq == std::string::npos) return false;
        name = c.substr(9, eq - 9);
        while (!name.empty() && name.back() == ' ') name.pop_back();
    } else {
        if (c.compare(8, 2, "= ") != 0) return false;
        name = c.substr(0, 8);
        while (!name.empty() && name.back() == ' ') name.pop_back();
        eq = 8;
    }
    std::string v = c.substr(eq + 1);
    size_t b = v.find_first_not_of(' ');
    if (b == std::string::npos) {
        value.clear();
    } else if (v[b] == '\'') {
        size_t e = v.find('\'', b + 1);
        value = v.substr(b + 1, e == std::string::npos ? std::string::npos : e - b - 1);
        while (!value.empty() && value.back() == ' ') value.pop_back();
    } else {
        size_t e = v.find('/', b);
        value = v.substr(b, e == std::string::npos ? std::string::npos : e - b);
        while (!value.empty() && value.back() == ' ') value.pop_back();
    }
    name = upper(name);
    return true;
}

void put_be64(unsigned char *p, double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    for (int k = 7; k >= 0; k--) {
        p[k] = (unsigned char)(u & 0xFFu);
        u >>= 8;
    }
}

double get_be64(const unsigned char *p) {
    uint64_t u = 0;
    for (int k = 0; k < 8; k++) u = (u << 8) | p[k];
    double v;
    std::memcpy(&v, &u, 8);
    return v;
}

bool write_at(FILE *fp, long off, const void *buf, size_t len) {
    return std::fseek(fp, off, SEEK_SET) == 0 && std::fwrite(buf, 1, len, fp) == len;
}

// Writes header cards + END padded to whole blocks at `off`; returns length.
long write_header(FILE *fp, long off, const std::vector<std::string> &cards, int &status) {
    std::string h;
    for (const std::string &c : cards) h += c;
    h += pad_card("END");
    h.resize(round_block((long)h.size()), ' ');
    if (!write_at(fp, off, h.data(), h.size())) status = WRITE_ERROR;
    return (long)h.size();
}

void flush_primary(fitsfile *f, int &status) {
    if (!f->primary_pending || status) return;
    Hdu &p = f->hdus[0];
    p.header_off = 0;
    p.header_len = write_header(f->fp, 0, f->primary_cards, status);
    p.data_off = p.header_len;
    f->primary_pending = false;
}

Hdu *find(fitsfile *f, const std::string &extname, int &status) {
    for (Hdu &h : f->hdus)
        if (!h.extname.empty() && upper(h.extname) == upper(extname)) return &h;
    status = BAD_HDU_NUM;
    return nullptr;
}

long row_offset(const Hdu &h, int col) {
    long o = 0;
    for (int c = 0; c < col; c++) o += 8 * h.cols[c].repeat;
    return o;
}

void set_primary_key(fitsfile *f, const std::string &name, const std::string &value, const std::string &comment,
                     int &status) {
    if (status) return;
    if (!f || !f->primary_pending) {
        status = STATE_ERROR;  // primary header already on disk
        return;
    }
    const std::string card = value_card(name, value, comment);
    const std::string key = upper(name);
    for (std::string &c : f->primary_cards) {
        std::string n, v;
        if (parse_card(c.data(), n, v) && n == key) {
            c = card;
            f->hdus[0].keys[key] = value;
            return;
        }
    }
    f->primary_cards.push_back(card);
    f->hdus[0].keys[key] = value;
}

}  // namespace

fitsfile *create(const std::string &path, int &status) {
    if (status) return nullptr;
    FILE *fp = std::fopen(path.c_str(), "w+b");
    if (!fp) {
        status = FILE_NOT_CREATED;
        return nullptr;
    }
    fitsfile *f = new fitsfile();
    f->fp = fp;
    f->writable = true;
    f->primary_pending = true;
    f->primary_cards = {value_card("SIMPLE", "T", "file conforms to FITS standard"),
                        value_card("BITPIX", "16", "number of bits per data pixel"),
                        value_card("NAXIS", "0", "number of data axes"),
                        value_card("EXTEND", "T", "FITS dataset may contain extensions")};
    f->hdus.emplace_back();
    return f;
}

fitsfile *open(const std::string &path, bool readwrite, int &status) {
    if (status) return nullptr;
    FILE *fp = std::fopen(path.c_str(), readwrite ? "r+b" : "rb");
    if (!fp) {
        status = FILE_NOT_OPENED;
        return nullptr;
    }
    fitsfile *f = new fitsfile();
    f->fp = fp;
    f->writable = readwrite;
    std::fseek(fp, 0, SEEK_END);
    const long size = std::ftell(fp);
    long off = 0;
    char card[kCard];
    while (off < size && !status) {
        Hdu h;
        h.header_off = off;
        long naxis = 0, naxis_len[3] = {0, 0, 0}, bitpix = 0, pcount = 0, tfields = 0;
        std::map<int, std::string> ttype, tform, tunit;
        bool end = false;
        long pos = off;
        while (!end) {
            if (std::fseek(fp, pos, SEEK_SET) != 0 || std::fread(card, 1, kCard, fp) != (size_t)kCard) {
                status = READ_ERROR;
                break;
            }
            if (std::strncmp(card, "END", 3) == 0 && card[3] == ' ') {
                end = true;
                pos += kCard;
                break;
            }
            std::string name, value;
            if (parse_card(card, name, value)) {
                h.keys[name] = value;
                if (name == "BITPIX") bitpix = std::atol(value.c_str());
                else if (name == "NAXIS") naxis = std::atol(value.c_str());
                else if (name == "NAXIS1") naxis_len[1] = std::atol(value.c_str());
                else if (name == "NAXIS2") {
                    naxis_len[2] = std::atol(value.c_str());
                    h.naxis2_card = pos;
                } else if (name == "PCOUNT") pcount = std::atol(value.c_str());
                else if (name == "TFIELDS") tfields = std::atol(value.c_str());
                else if (name == "EXTNAME") h.extname = value;
                else if (name.compare(0, 5, "TTYPE") == 0) ttype[std::atoi(name.c_str() + 5)] = value;
                else if (name.compare(0, 5, "TFORM") == 0) tform[std::atoi(name.c_str() + 5)] = value;
                else if (name.compare(0, 5, "TUNIT") == 0) tunit[std::atoi(name.c_str() + 5)] = value;
            }
            pos += kCard;
        }
        if (status) break;
        h.header_len = round_block(pos - off);
        h.data_off = off + h.header_len;
        long data = 0;
        if (naxis > 0) {
            data = std::labs(bitpix) / 8;
            for (int k = 1; k <= naxis && k <= 2; k++) data *= (k == 1 ? naxis_len[1] : naxis_len[2]);
            data += pcount;
        }
        if (!h.extname.empty() && tfields > 0) {
            h.naxis1 = naxis_len[1];
            h.naxis2 = naxis_len[2];
            for (int c = 1; c <= tfields; c++) {
                const std::string &tf = tform[c];
                const size_t d = tf.find('D');
                if (d == std::string::npos || tf.find_first_not_of(" 0123456789") != d) {
                    h.cols.clear();  // not an FP64-only table: skip it
                    break;
                }
                const long rep = d == 0 ? 1 : std::atol(tf.substr(0, d).c_str());
                h.cols.push_back({ttype[c], rep, tunit[c]});
            }
        }
        f->hdus.push_back(h);
        off = h.data_off + round_block(data);
    }
    if (status || f->hdus.empty()) {
        if (!status) status = BAD_HEADER;
        std::fclose(fp);
        delete f;
        return nullptr;
    }
    return f;
}

void flush(fitsfile *f, int &status) {
    if (!f) {
        status = STATE_ERROR;
        return;
    }
    if (f->writable) {
        flush_primary(f, status);
        if (std::fflush(f->fp) != 0 && !status) status = WRITE_ERROR;
    }
}

void close(fitsfile *f, int &status) {
    if (!f) return;
    flush(f, status);
    std::fclose(f->fp);
    delete f;
}

void write_key_long(fitsfile *f, const std::string &name, long value, const std::string &comment, int &status) {
    set_primary_key(f, name, std::to_string(value), comment, status);
}

void write_key_dbl(fitsfile *f, const std::string &name, double value, const std::string &comment,
                   int &status) {
    set_primary_key(f, name, fmt_dbl(value), comment, status);
}

long read_key_long(fitsfile *f, const std::string &name, int &status) {
    if (status) return 0;
    auto it = f->hdus[0].keys.find(upper(name));
    if (it == f->hdus[0].keys.end()) {
        status = KEY_NO_EXIST;
        return 0;
    }
    return std::atol(it->second.c_str());
}

double read_key_dbl(fitsfile *f, const std::string &name, int &status) {
    if (status) return 0.0;
    auto it = f->hdus[0].keys.find(upper(name));
    if (it == f->hdus[0].keys.end()) {
        status = KEY_NO_EXIST;
        return 0.0;
    }
    std::string v = it->second;
    for (char &c : v)
        if (c == 'D') c = 'E';  // FITS allows D exponents
    return std::strtod(v.c_str(), nullptr);
}

void create_table(fitsfile *f, const std::string &extname, const std::vector<Column> &cols, int &status) {
    if (status) return;
    if (!f || !f->writable || cols.empty()) {
        status = STATE_ERROR;
        return;
    }
    flush_primary(f, status);
    if (status) return;
    const Hdu &last = f->hdus.back();
    long off = last.data_off + round_block(last.naxis1 * last.naxis2);
    Hdu h;
    h.extname = extname;
    h.cols = cols;
    for (const Column &c : cols) h.naxis1 += 8 * c.repeat;
    std::vector<std::string> cards = {string_card("XTENSION", "BINTABLE"),
                                      value_card("BITPIX", "8", "8-bit bytes"),
                                      value_card("NAXIS", "2", "2-dimensional binary table"),
                                      value_card("NAXIS1", std::to_string(h.naxis1), "width of table in bytes"),
                                      value_card("NAXIS2", "0", "number of rows in table"),
                                      value_card("PCOUNT", "0", "size of special data area"),
                                      value_card("GCOUNT", "1", "one data group (required keyword)"),
                                      value_card("TFIELDS", std::to_string(cols.size()), "number of fields in each row")};
    for (size_t c = 0; c < cols.size(); c++) {
        const std::string k = std::to_string(c + 1);
        cards.push_back(string_card("TTYPE" + k, cols[c].name));
        cards.push_back(string_card("TFORM" + k, (cols[c].repeat == 1 ? "" : std::to_string(cols[c].repeat)) + "D"));
        cards.push_back(string_card("TUNIT" + k, cols[c].unit));
    }
    cards.push_back(string_card("EXTNAME", extname));
    h.header_off = off;
    h.naxis2_card = off + 4 * kCard;
    h.header_len = write_header(f->fp, off, cards, status);
    h.data_off = off + h.header_len;
    f->hdus.push_back(h);
}

void append_rows(fitsfile *f, const std::string &extname, long nrows, const std::vector<const double *> &cols,
                 int &status) {
    if (status) return;
    if (!f || !f->writable) {
        status = STATE_ERROR;
        return;
    }
    Hdu *h = find(f, extname, status);
    if (!h) return;
    if (h != &f->hdus.back() || cols.size() != h->cols.size() || h->naxis2_card < 0) {
        status = h->naxis2_card < 0 ? NOT_BTABLE : STATE_ERROR;
        return;
    }
    std::vector<unsigned char> buf((size_t)(h->naxis1 * nrows));
    for (long r = 0; r < nrows; r++) {
        unsigned char *row = buf.data() + r * h->naxis1;
        for (size_t c = 0; c < cols.size(); c++) {
            const long rep = h->cols[c].repeat;
            unsigned char *p = row + row_offset(*h, (int)c);
            for (long k = 0; k < rep; k++) put_be64(p + 8 * k, cols[c][r * rep + k]);
        }
    }
    const long old_bytes = h->naxis1 * h->naxis2;
    const long new_bytes = old_bytes + h->naxis1 * nrows;
    if (!write_at(f->fp, h->data_off + old_bytes, buf.data(), buf.size())) {
        status = WRITE_ERROR;
        return;
    }
    const long pad = round_block(new_bytes) - new_bytes;
    if (pad) {
        std::vector<unsigned char> z((size_t)pad, 0);
        if (std::fwrite(z.data(), 1, z.size(), f->fp) != z.size()) {
            status = WRITE_ERROR;
            return;
        }
    }
    h->naxis2 += nrows;
    const std::string card = value_card("NAXIS2", std::to_string(h->naxis2), "number of rows in table");
    if (!write_at(f->fp, h->naxis2_card, card.data(), kCard)) status = WRITE_ERROR;
}

long num_rows(fitsfile *f, const std::string &extname, int &status) {
    if (status) return 0;
    Hdu *h = find(f, extname, status);
    return h ? h->naxis2 : 0;
}

std::vector<double> read_cell(fitsfile *f, const std::string &extname, int col, long row, int &status) {
    std::vector<double> out;
    if (status) return out;
    Hdu *h = find(f, extname, status);
    if (!h) return out;
    if (col < 0 || col >= (int)h->cols.size()) {
        status = NOT_BTABLE;
        return out;
    }
    if (row < 0 || row >= h->naxis2) {
        status = BAD_ROW_NUM;
        return out;
    }
    const long rep = h->cols[col].repeat;
    std::vector<unsigned char> buf((size_t)(8 * rep));
    if (std::fseek(f->fp, h->data_off + row * h->naxis1 + row_offset(*h, col), SEEK_SET) != 0 ||
        std::fread(buf.data(), 1, buf.size(), f->fp) != buf.size()) {
        status = READ_ERROR;
        return out;
    }
    out.resize((size_t)rep);
    for (long k = 0; k < rep; k++) out[(size_t)k] = get_be64(buf.data() + 8 * k);
    return out;
}

std::vector<double> read_column(fitsfile *f, const std::string &extname, int col, int &status) {
    std::vector<double> out;
    const long rows = num_rows(f, extname, status);
    for (long r = 0; r < rows && !status; r++) {
        std::vector<double> v = read_cell(f, extname, col, r, status);
        out.insert(out.end(), v.begin(), v.end());
    }
    return out;
}

}  // namespace fits
}  // namespace demon_gb300
