// Delta files: a native reader of picca's two on-disk layouts and the
// projection of the deltas (host code).
//
// picca reads delta files through fitsio and builds one Python object per
// line of sight (py/picca/io.py:333-380, py/picca/data.py:376-620), then
// projects each forest in NumPy (py/picca/data.py:622-655). At 400k forests
// that host stage outlasts the GPU kernels. Here a file's bytes (already
// decompressed) are parsed in one pass into structure-of-arrays buffers:
//  * one BINTABLE per line of sight: header RA, DEC, Z, THING_ID / PLATE /
//    MJD / FIBERID (or LOS_ID), BLINDING; columns LOGLAM or LAMBDA, DELTA
//    (DELTA_BLIND when blinded), WEIGHT, CONT; kept when z_min < Z < z_max;
//  * image files: LAMBDA (or LOGLAM) image, DELTA / WEIGHT / CONT images
//    (one row per line of sight) and a METADATA table; kept when
//    z_min <= Z <= z_max, pixels with weight > 0.
// Values are converted to FP64 exactly (big-endian E / D / I / J / K). The
// projection reproduces NumPy's summation order (pairwise sums in blocks of
// eight, the algorithm of numpy's add.reduce for contiguous float64), so the
// projected deltas are bit-identical to the reference's. This file is host
// code only.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int64_t kBlock = 2880;

struct Card {
    std::string key, value;  // value: raw text (strings without quotes)
    bool is_string = false;
};

struct Hdu {
    std::vector<Card> cards;
    int64_t data_offset = 0, data_bytes = 0;

    const Card *find(const char *key) const {
        for (const Card &c : cards)
            if (c.key == key) return &c;
        return nullptr;
    }
    bool has(const char *key) const { return find(key) != nullptr; }
    bool get_int(const char *key, int64_t *out) const {
        const Card *c = find(key);
        if (!c || c->is_string) return false;
        char *end = nullptr;
        const long long v = strtoll(c->value.c_str(), &end, 10);
        if (end == c->value.c_str()) return false;
        *out = v;
        return true;
    }
    bool get_double(const char *key, double *out) const {
        const Card *c = find(key);
        if (!c || c->is_string) return false;
        std::string t = c->value;
        for (char &ch : t)
            if (ch == 'D' || ch == 'd') ch = 'E';
        char *end = nullptr;
        const double v = strtod(t.c_str(), &end);
        if (end == t.c_str()) return false;
        *out = v;
        return true;
    }
    std::string get_string(const char *key, const char *fallback) const {
        const Card *c = find(key);
        return (c && c->is_string) ? c->value : std::string(fallback);
    }
};

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && s[a] == ' ') ++a;
    while (b > a && s[b - 1] == ' ') --b;
    return s.substr(a, b - a);
}

// Parse one header starting at pos; returns false on malformed input.
bool parse_header(const uint8_t *buf, int64_t size, int64_t pos, Hdu *hdu, int64_t *next) {
    bool ended = false;
    int64_t p = pos;
    while (!ended) {
        if (p + kBlock > size) return false;
        for (int k = 0; k < kBlock / 80 && !ended; ++k) {
            const char *card = reinterpret_cast<const char *>(buf + p + 80 * k);
            std::string key = trim(std::string(card, 8));
            if (key == "END") {
                ended = true;
                break;
            }
            if (card[8] != '=' || card[9] != ' ') continue;
            std::string text(card + 10, 70);
            Card c;
            c.key = key;
            size_t i = 0;
            while (i < text.size() && text[i] == ' ') ++i;
            if (i < text.size() && text[i] == '\'') {
                std::string v;
                for (size_t j = i + 1; j < text.size(); ++j) {
                    if (text[j] == '\'') {
                        if (j + 1 < text.size() && text[j + 1] == '\'') {
                            v += '\'';
                            ++j;
                            continue;
                        }
                        break;
                    }
                    v += text[j];
                }
                while (!v.empty() && v.back() == ' ') v.pop_back();
                c.value = v;
                c.is_string = true;
            } else {
                const size_t slash = text.find('/', i);
                c.value = trim(text.substr(i, slash == std::string::npos ? std::string::npos
                                                                          : slash - i));
            }
            hdu->cards.push_back(c);
        }
        p += kBlock;
    }
    int64_t bitpix = 0, naxis = 0, pcount = 0, gcount = 1;
    if (!hdu->get_int("BITPIX", &bitpix) || !hdu->get_int("NAXIS", &naxis)) return false;
    hdu->get_int("PCOUNT", &pcount);
    hdu->get_int("GCOUNT", &gcount);
    int64_t count = naxis > 0 ? 1 : 0;
    for (int64_t a = 1; a <= naxis; ++a) {
        const std::string key = "NAXIS" + std::to_string(a);
        int64_t n = 0;
        if (!hdu->get_int(key.c_str(), &n) || n < 0) return false;
        count *= n;
    }
    const int64_t bytes = (bitpix < 0 ? -bitpix : bitpix) / 8 * gcount * (pcount + count);
    hdu->data_offset = p;
    hdu->data_bytes = naxis > 0 ? bytes : 0;
    *next = p + (hdu->data_bytes + kBlock - 1) / kBlock * kBlock;
    return *next <= size + kBlock && hdu->data_offset + hdu->data_bytes <= size;
}

bool parse_file(const uint8_t *buf, int64_t size, std::vector<Hdu> *hdus) {
    int64_t pos = 0;
    while (pos + kBlock <= size) {
        Hdu h;
        int64_t next = 0;
        if (!parse_header(buf, size, pos, &h, &next)) return false;
        hdus->push_back(std::move(h));
        pos = next;
    }
    return !hdus->empty();
}

uint64_t load_be(const uint8_t *p, int bytes) {
    uint64_t v = 0;
    for (int k = 0; k < bytes; ++k) v = (v << 8) | p[k];
    return v;
}

// A value of FITS type code `t` at p, as double / int64.
double read_double(const uint8_t *p, char t) {
    switch (t) {
        case 'E': {
            const uint32_t u = (uint32_t)load_be(p, 4);
            float f;
            memcpy(&f, &u, 4);
            return (double)f;
        }
        case 'D': {
            const uint64_t u = load_be(p, 8);
            double d;
            memcpy(&d, &u, 8);
            return d;
        }
        case 'I': return (double)(int16_t)load_be(p, 2);
        case 'J': return (double)(int32_t)load_be(p, 4);
        case 'K': return (double)(int64_t)load_be(p, 8);
        case 'B': return (double)p[0];
        default: return NAN;
    }
}
int64_t read_int(const uint8_t *p, char t) {
    switch (t) {
        case 'I': return (int16_t)load_be(p, 2);
        case 'J': return (int32_t)load_be(p, 4);
        case 'K': return (int64_t)load_be(p, 8);
        case 'B': return p[0];
        case 'E': return (int64_t)read_double(p, t);
        case 'D': return (int64_t)read_double(p, t);
        default: return 0;
    }
}

struct Column {
    std::string name;
    char type = 0;
    int64_t repeat = 1, offset = 0;
};

int type_bytes(char t) {
    switch (t) {
        case 'L': case 'B': case 'A': return 1;
        case 'I': return 2;
        case 'J': case 'E': return 4;
        case 'K': case 'D': return 8;
        case 'C': return 8;
        case 'M': return 16;
        default: return -1;
    }
}

bool table_columns(const Hdu &h, std::vector<Column> *cols, int64_t *row_bytes, int64_t *rows) {
    int64_t nf = 0;
    if (!h.get_int("TFIELDS", &nf) || !h.get_int("NAXIS1", row_bytes) ||
        !h.get_int("NAXIS2", rows))
        return false;
    int64_t off = 0;
    for (int64_t k = 1; k <= nf; ++k) {
        Column c;
        c.name = h.get_string(("TTYPE" + std::to_string(k)).c_str(), "");
        const std::string form = h.get_string(("TFORM" + std::to_string(k)).c_str(), "");
        size_t i = 0;
        while (i < form.size() && isdigit((unsigned char)form[i])) ++i;
        c.repeat = i ? atoll(form.substr(0, i).c_str()) : 1;
        if (i >= form.size()) return false;
        c.type = form[i];
        c.offset = off;
        int b = c.type == 'X' ? 0 : type_bytes(c.type);
        if (b < 0) return false;
        off += c.type == 'X' ? (c.repeat + 7) / 8 : c.repeat * b;
        for (char &ch : c.name) ch = (char)toupper((unsigned char)ch);
        cols->push_back(c);
    }
    return off == *row_bytes;
}

const Column *column(const std::vector<Column> &cols, const char *name) {
    for (const Column &c : cols)
        if (c.name == name) return &c;
    return nullptr;
}

std::string extname(const Hdu &h) { return h.get_string("EXTNAME", ""); }

}  // namespace

// Reads one delta file; with out->los_id == NULL only counts.
int read_delta_file(const uint8_t *buf, int64_t size, double z_min, double z_max,
                    pg_delta_arrays *out) {
    std::vector<Hdu> hdus;
    if (!parse_file(buf, size, &hdus)) return PG_ERR_INVALID_ARGUMENT;
    const bool fill = out->los_id != nullptr;
    int image = -1;
    for (size_t k = 1; k < hdus.size(); ++k)
        if (extname(hdus[k]) == "LAMBDA" || extname(hdus[k]) == "LOGLAM") image = (int)k;
    int64_t nlos = 0, npix = 0;
    out->format = image >= 0 ? 1 : 0;
    if (image < 0) {
        int wave_lambda = -1;
        for (size_t k = 1; k < hdus.size(); ++k) {
            const Hdu &h = hdus[k];
            double z = 0;
            if (!h.get_double("Z", &z)) return PG_ERR_INVALID_ARGUMENT;
            if (!(z_min < z && z < z_max)) continue;
            std::vector<Column> cols;
            int64_t row_bytes = 0, rows = 0;
            if (!table_columns(h, &cols, &row_bytes, &rows)) return PG_ERR_UNSUPPORTED;
            const std::string blinding = h.get_string("BLINDING", "none");
            const Column *cd = column(cols, blinding != "none" ? "DELTA_BLIND" : "DELTA");
            const Column *cl = column(cols, "LOGLAM");
            const int is_lambda = cl ? 0 : 1;
            if (!cl) cl = column(cols, "LAMBDA");
            const Column *cw = column(cols, "WEIGHT"), *cc = column(cols, "CONT");
            if (!cd || !cl || !cw || !cc) return PG_ERR_UNSUPPORTED;
            if (wave_lambda >= 0 && wave_lambda != is_lambda) return PG_ERR_UNSUPPORTED;
            wave_lambda = is_lambda;
            for (const Column *c : {cd, cl, cw, cc})
                if (c->repeat != 1 || (c->type != 'E' && c->type != 'D'))
                    return PG_ERR_UNSUPPORTED;
            if (fill) {
                int64_t los = 0;
                if (h.get_int("THING_ID", &los)) {
                    out->los_id[nlos] = los;
                    if (!h.get_int("PLATE", &out->plate[nlos]) ||
                        !h.get_int("MJD", &out->mjd[nlos]) ||
                        !h.get_int("FIBERID", &out->fiberid[nlos]))
                        return PG_ERR_INVALID_ARGUMENT;
                } else if (h.get_int("LOS_ID", &los)) {
                    out->los_id[nlos] = out->plate[nlos] = out->mjd[nlos] = out->fiberid[nlos] =
                        los;
                } else {
                    return PG_ERR_INVALID_ARGUMENT;
                }
                if (!h.get_double("RA", &out->ra[nlos]) || !h.get_double("DEC", &out->dec[nlos]))
                    return PG_ERR_INVALID_ARGUMENT;
                out->z_qso[nlos] = z;
                const uint8_t *base = buf + h.data_offset;
                for (int64_t r = 0; r < rows; ++r) {
                    const uint8_t *row = base + r * row_bytes;
                    const int64_t q = npix + r;
                    out->wave[q] = read_double(row + cl->offset, cl->type);
                    out->delta[q] = read_double(row + cd->offset, cd->type);
                    out->weights[q] = read_double(row + cw->offset, cw->type);
                    out->cont[q] = read_double(row + cc->offset, cc->type);
                }
                out->pix_offset[nlos + 1] = npix + rows;
            }
            npix += rows;
            ++nlos;
        }
        out->wave_is_lambda = wave_lambda > 0;
    } else {
        const Hdu *lam = &hdus[image], *dl = nullptr, *wt = nullptr, *ct = nullptr,
                  *meta = nullptr;
        for (size_t k = 1; k < hdus.size(); ++k)
            if (extname(hdus[k]) == "METADATA") meta = &hdus[k];
        if (!meta) return PG_ERR_INVALID_ARGUMENT;
        const std::string blinding = meta->get_string("BLINDING", "none");
        const std::string dname = blinding != "none" ? "DELTA_BLIND" : "DELTA";
        for (size_t k = 1; k < hdus.size(); ++k) {
            const std::string e = extname(hdus[k]);
            if (e == dname) dl = &hdus[k];
            if (e == "WEIGHT") wt = &hdus[k];
            if (e == "CONT") ct = &hdus[k];
        }
        if (!dl || !wt || !ct) return PG_ERR_UNSUPPORTED;
        out->wave_is_lambda = extname(*lam) == "LAMBDA";
        int64_t nwave = 0, bp = 0;
        if (!lam->get_int("NAXIS1", &nwave) || !lam->get_int("BITPIX", &bp)) return PG_ERR_INVALID_ARGUMENT;
        const char lt = bp == -64 ? 'D' : bp == -32 ? 'E' : 0;
        if (!lt) return PG_ERR_UNSUPPORTED;
        const Hdu *images[3] = {dl, wt, ct};
        char it[3];
        for (int k = 0; k < 3; ++k) {
            int64_t n1 = 0, n2 = 0, b = 0;
            if (!images[k]->get_int("NAXIS1", &n1) || !images[k]->get_int("NAXIS2", &n2) ||
                !images[k]->get_int("BITPIX", &b) || n1 != nwave)
                return PG_ERR_INVALID_ARGUMENT;
            it[k] = b == -64 ? 'D' : b == -32 ? 'E' : 0;
            if (!it[k]) return PG_ERR_UNSUPPORTED;
        }
        std::vector<Column> cols;
        int64_t row_bytes = 0, rows = 0;
        if (!table_columns(*meta, &cols, &row_bytes, &rows)) return PG_ERR_UNSUPPORTED;
        int64_t n2 = 0;
        wt->get_int("NAXIS2", &n2);
        if (n2 != rows) return PG_ERR_INVALID_ARGUMENT;
        const Column *cz = column(cols, "Z"), *cra = column(cols, "RA"), *cdec = column(cols, "DEC");
        const Column *cid = column(cols, "THING_ID");
        const Column *cpl = column(cols, "PLATE"), *cmj = column(cols, "MJD"),
                     *cfb = column(cols, "FIBERID");
        const bool thing = cid != nullptr;
        if (!thing) cid = column(cols, "LOS_ID");
        if (!cz || !cra || !cdec || !cid || (thing && (!cpl || !cmj || !cfb)))
            return PG_ERR_INVALID_ARGUMENT;
        // identifiers stored as text (coadded SDSS plates "3655-3657") are
        // left to the per-object reader
        for (const Column *c : {cid, cpl, cmj, cfb})
            if (c && (c->type == 'A' || c->repeat != 1)) return PG_ERR_UNSUPPORTED;
        const uint8_t *mrow0 = buf + meta->data_offset;
        const int eb = it[1] == 'D' ? 8 : 4;
        const int lb = lt == 'D' ? 8 : 4;
        for (int64_t r = 0; r < rows; ++r) {
            const uint8_t *mrow = mrow0 + r * row_bytes;
            const double z = read_double(mrow + cz->offset, cz->type);
            if (!(z_min <= z && z <= z_max)) continue;
            const uint8_t *wrow = buf + wt->data_offset + r * nwave * eb;
            int64_t kept = 0;
            for (int64_t p = 0; p < nwave; ++p) {
                const double w = read_double(wrow + p * eb, it[1]);
                if (!(w > 0)) continue;
                if (fill) {
                    const int64_t q = npix + kept;
                    const int db = it[0] == 'D' ? 8 : 4, cb = it[2] == 'D' ? 8 : 4;
                    out->weights[q] = w;
                    out->wave[q] = read_double(buf + lam->data_offset + p * lb, lt);
                    out->delta[q] = read_double(buf + dl->data_offset + (r * nwave + p) * db, it[0]);
                    out->cont[q] = read_double(buf + ct->data_offset + (r * nwave + p) * cb, it[2]);
                }
                ++kept;
            }
            if (fill) {
                out->los_id[nlos] = read_int(mrow + cid->offset, cid->type);
                if (thing) {
                    out->plate[nlos] = read_int(mrow + cpl->offset, cpl->type);
                    out->mjd[nlos] = read_int(mrow + cmj->offset, cmj->type);
                    out->fiberid[nlos] = read_int(mrow + cfb->offset, cfb->type);
                } else {
                    out->plate[nlos] = out->mjd[nlos] = out->fiberid[nlos] = out->los_id[nlos];
                }
                out->ra[nlos] = read_double(mrow + cra->offset, cra->type);
                out->dec[nlos] = read_double(mrow + cdec->offset, cdec->type);
                out->z_qso[nlos] = z;
                out->pix_offset[nlos + 1] = npix + kept;
            }
            npix += kept;
            ++nlos;
        }
    }
    if (fill) out->pix_offset[0] = 0;
    out->num_los = nlos;
    out->num_pixels = npix;
    return PG_OK;
}

namespace {

// numpy's pairwise sum of n contiguous doubles (add.reduce, float64).
double np_pairwise(const double *a, int64_t n) {
    if (n < 8) {
        double r = 0.;
        for (int64_t i = 0; i < n; ++i) r += a[i];
        return r;
    }
    if (n <= 128) {
        double r[8];
        for (int k = 0; k < 8; ++k) r[k] = a[k];
        int64_t i = 8;
        for (; i < n - (n % 8); i += 8)
            for (int k = 0; k < 8; ++k) r[k] += a[i + k];
        double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; ++i) res += a[i];
        return res;
    }
    int64_t n2 = n / 2;
    n2 -= n2 % 8;
    return np_pairwise(a, n2) + np_pairwise(a + n2, n - n2);
}

double np_sum(const double *a, int64_t n) { return 0. + np_pairwise(a, n); }

// Delta.project (py/picca/data.py:622-655) with NumPy's operation order.
void project_one(int64_t n, const double *ll, const double *w, double *d, int order,
                 std::vector<double> &t1, std::vector<double> &t2) {
    t1.resize(n);
    t2.resize(n);
    const double sum_w = np_sum(w, n);
    if (!(sum_w > 0.)) return;
    for (int64_t i = 0; i < n; ++i) t1[i] = d[i] * w[i];
    const double mean_delta = np_sum(t1.data(), n) / sum_w;
    if (order == 1 && n > 1) {
        for (int64_t i = 0; i < n; ++i) t1[i] = ll[i] * w[i];
        const double mean_ll = np_sum(t1.data(), n) / sum_w;
        for (int64_t i = 0; i < n; ++i) t2[i] = ll[i] - mean_ll;  // meanless log lambda
        for (int64_t i = 0; i < n; ++i) t1[i] = (w[i] * d[i]) * t2[i];
        const double num = np_sum(t1.data(), n);
        for (int64_t i = 0; i < n; ++i) t1[i] = w[i] * (t2[i] * t2[i]);
        const double slope = num / np_sum(t1.data(), n);
        for (int64_t i = 0; i < n; ++i) d[i] = d[i] - (mean_delta + slope * t2[i]);
    } else if (order == 1) {
        for (int64_t i = 0; i < n; ++i) d[i] = d[i] - (mean_delta + d[i]);
    } else {
        for (int64_t i = 0; i < n; ++i) d[i] = d[i] - (mean_delta + 0.);
    }
}

}  // namespace

int project_deltas(int64_t num_los, const int64_t *pix_offset, const double *log_lambda,
                   const double *weights, double *delta, const int32_t *order, int threads) {
    if (num_los <= 0) return PG_OK;
    threads = std::max(1, std::min<int>(threads, (int)std::min<int64_t>(num_los, 256)));
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([=]() {
            std::vector<double> t1, t2;
            for (int64_t f = t; f < num_los; f += threads) {
                const int64_t o = pix_offset[f], n = pix_offset[f + 1] - o;
                project_one(n, log_lambda + o, weights + o, delta + o, order[f], t1, t2);
            }
        });
    }
    for (auto &th : pool) th.join();
    return PG_OK;
}

}  // namespace pg
