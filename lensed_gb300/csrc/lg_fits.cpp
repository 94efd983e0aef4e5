// FITS output without CFITSIO: an empty primary HDU followed by one 2-D
// float32 IMAGE extension per layer, each named by EXTNAME.  This is the
// file layout the reference writes through CFITSIO in write_fits
// (src/data.c:129-165), used by write_output (src/data.c:372-391, a file)
// and write_memory (src/data.c:393-419, a memory block).
//
// Header cards follow the FITS 4.0 fixed format: keyword in columns 1-8,
// "= " in 9-10, logical and integer values right-justified to column 30,
// string values quoted from column 11 and padded to at least 8 characters.
// Headers are padded with blanks and data with zeros to 2880-byte records;
// pixels are big-endian IEEE float32, rows of `width` pixels from the bottom
// row up (pixel index x + width*y).

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>

#include "lg_internal.h"

namespace {

constexpr size_t kRecord = 2880;

struct Header {
    std::string s;

    void card(const std::string& key, const std::string& value, const std::string& comment)
    {
        std::string c = key;
        c.resize(8, ' ');
        c += "= ";
        c += value;
        if (!comment.empty()) c += " / " + comment;
        c.resize(80, ' ');
        s += c;
    }
    void logical(const char* key, bool v, const char* comment)
    {
        std::string val(20, ' ');
        val[19] = v ? 'T' : 'F';
        card(key, val, comment);
    }
    void integer(const char* key, long long v, const char* comment)
    {
        char b[32];
        std::snprintf(b, sizeof b, "%20lld", v);
        card(key, b, comment);
    }
    void string(const char* key, const std::string& v, const char* comment)
    {
        std::string q = "'";
        for (char ch : v) {
            q += ch;
            if (ch == '\'') q += '\'';
        }
        while (q.size() < 9) q += ' ';
        q += '\'';
        card(key, q, comment);
    }
    void comment(const std::string& text)
    {
        std::string c = "COMMENT " + text;
        c.resize(80, ' ');
        s += c;
    }
    void end()
    {
        std::string c = "END";
        c.resize(80, ' ');
        s += c;
        s.resize((s.size() + kRecord - 1) / kRecord * kRecord, ' ');
    }
};

bool printable(const char* t, size_t max_len)
{
    size_t n = 0;
    for (; t[n]; ++n) {
        const unsigned char ch = (unsigned char)t[n];
        if (ch < 0x20 || ch > 0x7e || n >= max_len) return false;
    }
    return true;
}

std::string utc_date()
{
    std::time_t now = std::time(nullptr);
    std::tm tm{};
    gmtime_r(&now, &tm);
    char b[32];
    std::strftime(b, sizeof b, "%Y-%m-%dT%H:%M:%S", &tm);
    return b;
}

int build(int width, int height, int n, const float* const* layers, const char* const* names, std::string& out)
{
    if (width <= 0 || height <= 0 || n < 0 || (n > 0 && !layers)) {
        lg::set_global_error("write_fits: invalid image size or layer list");
        return LG_ERR_INPUT;
    }
    for (int i = 0; i < n; ++i) {
        if (!layers[i]) {
            lg::set_global_error("write_fits: NULL layer");
            return LG_ERR_INPUT;
        }
        // an EXTNAME value must fit one 80-column card
        if (names && names[i] && !printable(names[i], 68)) {
            lg::set_global_error("write_fits: extension names must be printable ASCII, at most 68 characters");
            return LG_ERR_INPUT;
        }
    }
    const size_t npix = (size_t)width * (size_t)height;
    const size_t data = (npix * 4 + kRecord - 1) / kRecord * kRecord;
    out.clear();
    out.reserve(kRecord * (1 + 2 * (size_t)n) + data * (size_t)n);

    Header p;
    p.logical("SIMPLE", true, "file does conform to FITS standard");
    p.integer("BITPIX", 16, "number of bits per data pixel");
    p.integer("NAXIS", 0, "number of data axes");
    p.logical("EXTEND", true, "FITS dataset may contain extensions");
    p.string("ORIGIN", lg_version(), "FITS file originator");
    p.comment("IMG model, RES residuals, RAW unconvolved model, ERR relative");
    p.comment("quadrature error, WHT weight, PVL per-pixel chi^2 p-value");
    p.string("DATE", utc_date(), "file creation date (YYYY-MM-DDThh:mm:ss UT)");
    p.end();
    out += p.s;

    for (int i = 0; i < n; ++i) {
        Header h;
        h.string("XTENSION", "IMAGE", "IMAGE extension");
        h.integer("BITPIX", -32, "number of bits per data pixel");
        h.integer("NAXIS", 2, "number of data axes");
        h.integer("NAXIS1", width, "length of data axis 1");
        h.integer("NAXIS2", height, "length of data axis 2");
        h.integer("PCOUNT", 0, "required keyword; must = 0");
        h.integer("GCOUNT", 1, "required keyword; must = 1");
        if (names && names[i]) h.string("EXTNAME", names[i], "extension name");
        h.end();
        out += h.s;
        const size_t at = out.size();
        out.resize(at + data, '\0');
        unsigned char* d = reinterpret_cast<unsigned char*>(&out[at]);
        for (size_t k = 0; k < npix; ++k) {
            uint32_t u;
            std::memcpy(&u, &layers[i][k], 4);
            d[4 * k + 0] = (unsigned char)(u >> 24);
            d[4 * k + 1] = (unsigned char)(u >> 16);
            d[4 * k + 2] = (unsigned char)(u >> 8);
            d[4 * k + 3] = (unsigned char)u;
        }
    }
    return LG_OK;
}

}  // namespace

extern "C" int lg_write_fits_memory(int width, int height, int nlayers, const float* const* layers,
                                    const char* const* names, void* buf, size_t capacity, size_t* size)
{
    std::string out;
    int rc = build(width, height, nlayers, layers, names, out);
    if (rc) return rc;
    if (size) *size = out.size();
    if (!buf) return LG_OK;
    if (capacity < out.size()) {
        lg::set_global_error("write_fits_memory: buffer too small");
        return LG_ERR_INPUT;
    }
    std::memcpy(buf, out.data(), out.size());
    return LG_OK;
}

extern "C" int lg_write_fits(const char* path, int width, int height, int nlayers, const float* const* layers,
                             const char* const* names)
{
    if (!path) {
        lg::set_global_error("write_fits: no file name");
        return LG_ERR_INPUT;
    }
    std::string out;
    int rc = build(width, height, nlayers, layers, names, out);
    if (rc) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        lg::set_global_error((std::string("write_fits: cannot create ") + path).c_str());
        return LG_ERR_INPUT;
    }
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    if (std::fclose(f) != 0 || !ok) {
        lg::set_global_error((std::string("write_fits: write failed for ") + path).c_str());
        return LG_ERR_INPUT;
    }
    return LG_OK;
}
