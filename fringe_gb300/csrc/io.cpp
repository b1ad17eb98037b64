// io.cpp -- file-level module call (fpl_process), mirroring evd_process.
//
// Reads the inputs the reference's evd / phase_link modules read through
// GDAL, without GDAL:
//   * the stack: a VRT whose bands carry a "Date" item in metadata domain
//     "slc" (written by python/tops2vrt.py:198-216), each band a SimpleSource
//     over a per-date VRT with a VRTRawRasterBand (tops2vrt.py:143-151), an
//     ENVI file, or a raw CFloat32 file;
//   * the weights (nmap): an ENVI UInt32 file with nulong bands, interleave
//     BIP, and HALFWINDOWX / HALFWINDOWY in its header
//     (src/nmap/nmap.cpp:235-262,588-591);
// and writes the reference's outputs (src/evd/evd.cpp:266-366): one ENVI
// CFloat32 file per date named <date>.slc, tcorr.bin (Float32) and the
// compressed SLC (CFloat32), each with a "<name>.hdr" header.
// Rows are processed in blocks with the reference's block / halo logic
// (src/evd/evd.cpp:169-187,399-443,861-870); each block runs on the GPU via
// fpl_run.  Return codes are the reference's (101-121).
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "fringe_gb300.h"
#include "guard.h"

namespace {

// ---------------------------------------------------------------- strings
std::string lower(std::string s)
{
    for (auto &c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}
std::string trim(const std::string &s)
{
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}
std::string dirname_of(const std::string &p)
{
    size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}
std::string join_path(const std::string &d, const std::string &f)
{
    if (f.empty() || f[0] == '/') return f;
    if (d.empty()) return f;
    return d + "/" + f;
}
bool read_text(const std::string &path, std::string &out)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out.resize(n > 0 ? (size_t)n : 0);
    size_t got = n > 0 ? std::fread(&out[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == out.size();
}
bool file_exists(const std::string &p)
{
    struct stat st;
    return ::stat(p.c_str(), &st) == 0;
}

// ------------------------------------------------------------- tiny XML
// Enough for GDAL-written VRTs: elements with attributes and text bodies.
struct XmlElem {
    std::string tag;
    std::string attrs;   // raw attribute text
    std::string body;    // raw inner text
};

// all elements <tag ...>...</tag> (case-insensitive tag) directly in text
std::vector<XmlElem> xml_find(const std::string &text, const std::string &tag)
{
    std::vector<XmlElem> out;
    const std::string lt = lower(text), ltag = lower(tag);
    size_t pos = 0;
    while (true) {
        size_t a = lt.find("<" + ltag, pos);
        if (a == std::string::npos) break;
        size_t after = a + 1 + ltag.size();
        if (after < lt.size() && !(std::isspace((unsigned char)lt[after]) || lt[after] == '>' || lt[after] == '/')) {
            pos = after;
            continue;
        }
        size_t gt = lt.find('>', after);
        if (gt == std::string::npos) break;
        XmlElem e;
        e.tag = tag;
        e.attrs = text.substr(after, gt - after);
        if (gt > 0 && lt[gt - 1] == '/') {   // self-closing
            out.push_back(e);
            pos = gt + 1;
            continue;
        }
        // matching close tag, allowing nested elements of the same name
        int depth = 1;
        size_t p = gt + 1, body_end = std::string::npos;
        while (depth > 0) {
            size_t o = lt.find("<" + ltag, p), c = lt.find("</" + ltag, p);
            if (c == std::string::npos) break;
            if (o != std::string::npos && o < c) {
                size_t oa = o + 1 + ltag.size();
                if (oa < lt.size() && (std::isspace((unsigned char)lt[oa]) || lt[oa] == '>')) depth++;
                p = oa;
            } else {
                depth--;
                if (depth == 0) body_end = c;
                p = c + 2 + ltag.size();
            }
        }
        if (body_end == std::string::npos) break;
        e.body = text.substr(gt + 1, body_end - gt - 1);
        out.push_back(e);
        pos = lt.find('>', body_end) + 1;
    }
    return out;
}
bool xml_attr(const std::string &attrs, const std::string &name, std::string &val)
{
    const std::string la = lower(attrs), ln = lower(name);
    size_t k = 0;
    while ((k = la.find(ln, k)) != std::string::npos) {
        bool start_ok = k == 0 || std::isspace((unsigned char)la[k - 1]);
        size_t e = k + ln.size();
        while (e < la.size() && std::isspace((unsigned char)la[e])) e++;
        if (start_ok && e < la.size() && la[e] == '=') {
            e++;
            while (e < la.size() && std::isspace((unsigned char)la[e])) e++;
            if (e < la.size() && (la[e] == '"' || la[e] == '\'')) {
                char q = la[e];
                size_t f = la.find(q, e + 1);
                if (f == std::string::npos) return false;
                val = attrs.substr(e + 1, f - e - 1);
                return true;
            }
        }
        k += ln.size();
    }
    return false;
}
std::string xml_text(const std::string &body, const std::string &tag, bool *found = nullptr,
                     std::string *attrs = nullptr)
{
    auto v = xml_find(body, tag);
    if (found) *found = !v.empty();
    if (v.empty()) return std::string();
    if (attrs) *attrs = v[0].attrs;
    return trim(v[0].body);
}

// ---------------------------------------------------------------- rasters
// A band of raw pixels: byte offset of pixel (x, y) is
// image_offset + y * line_offset + x * pixel_offset.
struct RawBand {
    std::string path;
    long long image_offset = 0, pixel_offset = 0, line_offset = 0;
    int bytes = 8;               // bytes per pixel value
    bool little = true;
    int xoff = 0, yoff = 0;      // window offset applied by a VRT SrcRect
};

struct EnviHeader {
    int samples = 0, lines = 0, bands = 0, data_type = 0, byte_order = 0;
    long long header_offset = 0;
    std::string interleave = "bsq";
    std::vector<std::pair<std::string, std::string>> items;   // lower-cased keys
};

bool parse_envi_header(const std::string &hdr_path, EnviHeader &h)
{
    std::string t;
    if (!read_text(hdr_path, t)) return false;
    if (lower(t).find("envi") != 0) return false;
    // join multi-line {...} values
    size_t pos = 0;
    while (pos < t.size()) {
        size_t eol = t.find('\n', pos);
        std::string line = t.substr(pos, eol == std::string::npos ? std::string::npos : eol - pos);
        pos = eol == std::string::npos ? t.size() : eol + 1;
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = lower(trim(line.substr(0, eq)));
        std::string val = trim(line.substr(eq + 1));
        if (!val.empty() && val[0] == '{') {
            while (val.find('}') == std::string::npos && pos < t.size()) {
                size_t e2 = t.find('\n', pos);
                val += " " + trim(t.substr(pos, e2 == std::string::npos ? std::string::npos : e2 - pos));
                pos = e2 == std::string::npos ? t.size() : e2 + 1;
            }
        }
        h.items.push_back({key, val});
        if (key == "samples") h.samples = std::atoi(val.c_str());
        else if (key == "lines") h.lines = std::atoi(val.c_str());
        else if (key == "bands") h.bands = std::atoi(val.c_str());
        else if (key == "data type") h.data_type = std::atoi(val.c_str());
        else if (key == "byte order") h.byte_order = std::atoi(val.c_str());
        else if (key == "header offset") h.header_offset = std::atoll(val.c_str());
        else if (key == "interleave") h.interleave = lower(val);
    }
    return h.samples > 0 && h.lines > 0 && h.bands > 0;
}

int envi_type_bytes(int dt)
{
    switch (dt) {
    case 1: return 1;
    case 2: case 12: return 2;
    case 3: case 4: case 13: return 4;
    case 5: case 6: case 14: case 15: return 8;
    case 9: return 16;
    }
    return 0;
}

std::string find_envi_header(const std::string &data_path)
{
    if (file_exists(data_path + ".hdr")) return data_path + ".hdr";
    size_t dot = data_path.find_last_of('.'), slash = data_path.find_last_of('/');
    if (dot != std::string::npos && (slash == std::string::npos || dot > slash)) {
        std::string alt = data_path.substr(0, dot) + ".hdr";
        if (file_exists(alt)) return alt;
    }
    return std::string();
}

bool envi_band(const std::string &data_path, const EnviHeader &h, int band, RawBand &rb)
{
    const int b = envi_type_bytes(h.data_type);
    if (!b || band < 0 || band >= h.bands) return false;
    rb.path = data_path;
    rb.bytes = b;
    rb.little = h.byte_order == 0;
    const long long W = h.samples, H = h.lines, B = h.bands;
    if (h.interleave == "bip") {
        rb.pixel_offset = B * b;
        rb.line_offset = W * B * b;
        rb.image_offset = h.header_offset + band * b;
    } else if (h.interleave == "bil") {
        rb.pixel_offset = b;
        rb.line_offset = W * B * b;
        rb.image_offset = h.header_offset + band * W * b;
    } else {
        rb.pixel_offset = b;
        rb.line_offset = W * b;
        rb.image_offset = h.header_offset + band * W * H * b;
    }
    return true;
}

// Resolves band `band` (0-based) of a dataset file (VRT or ENVI) to raw bytes.
bool resolve_band(const std::string &path, int band, RawBand &rb, int depth = 0);

bool resolve_vrt_band(const std::string &vrt_path, const std::string &text, int band, RawBand &rb, int depth)
{
    auto bands = xml_find(text, "VRTRasterBand");
    const XmlElem *eb = nullptr;
    for (auto &e : bands) {
        std::string bs;
        int bnum = xml_attr(e.attrs, "band", bs) ? std::atoi(bs.c_str()) : (int)(&e - &bands[0]) + 1;
        if (bnum == band + 1) { eb = &e; break; }
    }
    if (!eb) return false;
    std::string sub;
    const std::string dir = dirname_of(vrt_path);
    if (xml_attr(eb->attrs, "subClass", sub) && lower(sub) == "vrtrawrasterband") {
        std::string fattrs;
        bool f;
        std::string fn = xml_text(eb->body, "SourceFilename", &f, &fattrs);
        if (!f) return false;
        std::string rel;
        if (xml_attr(fattrs, "relativeToVRT", rel) && rel == "1") fn = join_path(dir, fn);
        rb.path = fn;
        rb.image_offset = std::atoll(xml_text(eb->body, "ImageOffset").c_str());
        rb.pixel_offset = std::atoll(xml_text(eb->body, "PixelOffset").c_str());
        rb.line_offset = std::atoll(xml_text(eb->body, "LineOffset").c_str());
        std::string bo = lower(xml_text(eb->body, "ByteOrder"));
        rb.little = bo.empty() || bo == "lsb";
        std::string dt;
        xml_attr(eb->attrs, "dataType", dt);
        dt = lower(dt);
        rb.bytes = dt == "cfloat32" ? 8 : (dt == "float32" || dt == "uint32" || dt == "int32") ? 4 : 8;
        rb.xoff = rb.yoff = 0;
        return true;
    }
    for (const char *st : {"SimpleSource", "ComplexSource"}) {
        auto srcs = xml_find(eb->body, st);
        if (srcs.empty()) continue;
        const std::string &sb = srcs[0].body;
        std::string fattrs;
        bool f;
        std::string fn = xml_text(sb, "SourceFilename", &f, &fattrs);
        if (!f) return false;
        std::string rel;
        if (xml_attr(fattrs, "relativeToVRT", rel) && rel == "1") fn = join_path(dir, fn);
        int sband = 1;
        bool fb;
        std::string sbs = xml_text(sb, "SourceBand", &fb);
        if (fb) sband = std::atoi(sbs.c_str());
        if (!resolve_band(fn, sband - 1, rb, depth + 1)) return false;
        auto src_rect = xml_find(sb, "SrcRect");
        if (!src_rect.empty()) {
            std::string xo, yo;
            if (xml_attr(src_rect[0].attrs, "xOff", xo)) rb.xoff += std::atoi(xo.c_str());
            if (xml_attr(src_rect[0].attrs, "yOff", yo)) rb.yoff += std::atoi(yo.c_str());
        }
        return true;
    }
    return false;
}

bool resolve_band(const std::string &path, int band, RawBand &rb, int depth)
{
    if (depth > 8) return false;
    std::string text;
    if (lower(path).size() >= 4 && lower(path).substr(lower(path).size() - 4) == ".vrt") {
        if (!read_text(path, text)) return false;
        return resolve_vrt_band(path, text, band, rb, depth);
    }
    std::string hdr = find_envi_header(path);
    if (!hdr.empty()) {
        EnviHeader h;
        if (!parse_envi_header(hdr, h)) return false;
        return envi_band(path, h, band, rb);
    }
    // a VRT without the .vrt suffix
    if (read_text(path, text) && lower(text).find("<vrtdataset") != std::string::npos)
        return resolve_vrt_band(path, text, band, rb, depth);
    return false;
}

// Reads rows [y0, y0+ny) x cols [0, w) of a raw band into dst (w*ny values of rb.bytes).
bool read_rows(const RawBand &rb, int w, int y0, int ny, void *dst)
{
    FILE *f = std::fopen(rb.path.c_str(), "rb");
    if (!f) return false;
    unsigned char *out = static_cast<unsigned char *>(dst);
    const long long ps = rb.pixel_offset, b = rb.bytes;
    std::vector<unsigned char> line;
    bool ok = true;
    for (int y = 0; y < ny && ok; ++y) {
        long long off = rb.image_offset + (long long)(y0 + y + rb.yoff) * rb.line_offset + (long long)rb.xoff * ps;
        if (std::fseek(f, off, SEEK_SET) != 0) { ok = false; break; }
        unsigned char *o = out + (size_t)y * w * b;
        if (ps == b) {
            ok = std::fread(o, 1, (size_t)w * b, f) == (size_t)w * b;
        } else {
            line.resize((size_t)(w - 1) * ps + b);
            ok = std::fread(line.data(), 1, line.size(), f) == line.size();
            for (int x = 0; ok && x < w; ++x) std::memcpy(o + (size_t)x * b, line.data() + (size_t)x * ps, b);
        }
        if (ok && !rb.little) {   // byte-swap each 4-byte word
            for (size_t k = 0; k + 4 <= (size_t)w * b; k += 4) {
                std::swap(o[k], o[k + 3]);
                std::swap(o[k + 1], o[k + 2]);
            }
        }
    }
    std::fclose(f);
    return ok;
}

// ------------------------------------------------------------- outputs
bool write_envi_header(const std::string &data_path, int cols, int rows, int bands, int dtype,
                       const char *desc)
{
    FILE *f = std::fopen((data_path + ".hdr").c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "ENVI\ndescription = {%s}\nsamples = %d\nlines = %d\nbands = %d\n"
                    "header offset = 0\nfile type = ENVI Standard\ndata type = %d\n"
                    "interleave = bip\nbyte order = 0\n",
                 desc, cols, rows, bands, dtype);
    std::fclose(f);
    return true;
}

struct OutFile {
    FILE *f = nullptr;
    ~OutFile() { if (f) std::fclose(f); }
};

bool create_output(const std::string &path, int cols, int rows, int bytes, int dtype, OutFile &of)
{
    of.f = std::fopen(path.c_str(), "wb+");
    if (!of.f) return false;
    // size the file (zeros for rows no block writes)
    if (rows > 0 && cols > 0) {
        long long total = (long long)rows * cols * bytes;
        if (std::fseek(of.f, total - 1, SEEK_SET) != 0 || std::fputc(0, of.f) == EOF) return false;
    }
    return write_envi_header(path, cols, rows, 1, dtype, path.c_str());
}

bool write_rows(OutFile &of, int cols, int bytes, int y0, int ny, const void *src)
{
    if (std::fseek(of.f, (long long)y0 * cols * bytes, SEEK_SET) != 0) return false;
    size_t n = (size_t)ny * cols * bytes;
    return std::fwrite(src, 1, n, of.f) == n;
}

}  // namespace

extern "C" {

void fpl_options_default(fpl_options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    // evdOptions::evdOptions, src/evd/evd.hpp:58-68
    o->blocksize = 64;
    o->memsize = 2048;
    o->Nx = 5;
    o->Ny = 5;
    o->minNeighbors = 2;
    o->miniStackCount = 1;
    o->method = "MLE";
    o->bandWidth = -1;
    o->semantics = FPL_SEM_EVD;
    o->precision = FPL_PREC_FP32;
    o->device = 0;
    o->verbose = 1;
}

int fpl_process(const fpl_options *opts)
{
    return fpl_guard([&]() -> int {
        if (!opts || !opts->inputDS || !opts->wtsDS || !opts->outputFolder) return FPL_ERR_OPTIONS;
        const bool verbose = opts->verbose != 0;
        const std::string method = opts->method ? opts->method : "MLE";
        int meth;
        if (method == "MLE") meth = FPL_METHOD_MLE;
        else if (method == "EVD") meth = FPL_METHOD_EVD;
        else if (method == "STBAS") meth = FPL_METHOD_STBAS;
        else return FPL_ERR_OPTIONS;
        const int Ny = opts->Ny, Nx = opts->Nx;
        const int nulong = (int)std::ceil(((2 * Ny + 1) * (2 * Nx + 1)) / 32.0);   // evd.cpp:47-48

        // ---- stack (evd.cpp:51-71) ----
        std::string vrt;
        std::string in = opts->inputDS;
        if (!read_text(in, vrt) || lower(vrt).find("<vrtdataset") == std::string::npos) {
            if (verbose) std::printf("Cannot open stack file { %s } for reading (a VRT is expected)\n", in.c_str());
            return FPL_ERR_OPEN_STACK;
        }
        auto ds = xml_find(vrt, "VRTDataset");
        std::string xs, ys;
        if (ds.empty() || !xml_attr(ds[0].attrs, "rasterXSize", xs) || !xml_attr(ds[0].attrs, "rasterYSize", ys))
            return FPL_ERR_OPEN_STACK;
        const int cols = std::atoi(xs.c_str()), rows = std::atoi(ys.c_str());
        const int nbands = (int)xml_find(vrt, "VRTRasterBand").size();
        if (cols <= 0 || rows <= 0 || nbands <= 0) return FPL_ERR_OPEN_STACK;
        if (verbose) std::printf("Number of rows  = %d\nNumber of cols  = %d\nNumber of bands = %d\n", rows, cols, nbands);

        // ---- STBAS bandwidth (evd.cpp:74-91) ----
        if (meth == FPL_METHOD_STBAS) {
            if (opts->bandWidth <= 0 || opts->bandWidth >= nbands - 1) return FPL_ERR_OPTIONS;
        }
        if (opts->miniStackCount < 1 || opts->miniStackCount > nbands) return FPL_ERR_OPTIONS;
        if (nbands > FPL_MAX_BANDS || nulong > FPL_MAX_NULONG) return FPL_ERR_UNSUPPORTED;

        // ---- weights (evd.cpp:93-166) ----
        std::string wts = opts->wtsDS;
        std::string whdr = find_envi_header(wts);
        EnviHeader wh;
        if (whdr.empty() || !parse_envi_header(whdr, wh)) {
            if (verbose) std::printf("Could not open weights dataset {%s}\n", wts.c_str());
            return FPL_ERR_OPEN_WEIGHTS;
        }
        {
            int code = 0;
            if (wh.samples != cols) code = FPL_ERR_WIDTH;
            if (wh.lines != rows) code = FPL_ERR_LENGTH;
            if (wh.bands != nulong) code = FPL_ERR_NULONG;
            int inNx = 0, inNy = 0;
            for (auto &kv : wh.items) {
                if (kv.first == "halfwindowx") inNx = std::atoi(kv.second.c_str());
                if (kv.first == "halfwindowy") inNy = std::atoi(kv.second.c_str());
            }
            if (inNx != Nx || inNx == 0) code = FPL_ERR_HALFWINDOWX;
            if (inNy != Ny || inNy == 0) code = FPL_ERR_HALFWINDOWY;
            if (envi_type_bytes(wh.data_type) != 4) code = code ? code : FPL_ERR_OPEN_WEIGHTS;
            if (code) {
                if (verbose) std::printf("Exiting with error code ....(%d)\n", code);
                return code;
            }
        }
        std::vector<RawBand> wband(1);
        // nulong words per pixel, interleaved: read them as one BIP "band" of nulong*4 bytes
        if (!envi_band(wts, wh, 0, wband[0])) return FPL_ERR_OPEN_WEIGHTS;
        if (lower(wh.interleave) != "bip") {
            if (verbose) std::printf("Weights dataset must be BIP interleaved\n");
            return FPL_ERR_OPEN_WEIGHTS;
        }
        wband[0].bytes = 4 * nulong;
        wband[0].pixel_offset = 4LL * nulong;

        // ---- dates (evd.cpp:210-223) and band sources ----
        std::vector<std::string> dates(nbands);
        std::vector<RawBand> bands(nbands);
        {
            auto vb = xml_find(vrt, "VRTRasterBand");
            for (int b = 0; b < nbands; ++b) {
                std::string date;
                for (auto &md : xml_find(vb[b].body, "Metadata")) {
                    std::string dom;
                    if (!xml_attr(md.attrs, "domain", dom) || dom != "slc") continue;
                    for (auto &mdi : xml_find(md.body, "MDI")) {
                        std::string key;
                        if (xml_attr(mdi.attrs, "key", key) && key == "Date") date = trim(mdi.body);
                    }
                }
                if (date.size() != 8) {
                    if (verbose) std::printf("Band %d does not appear to have Date information in slc metadata domain \n", b + 1);
                    return FPL_ERR_DATE;
                }
                dates[b] = date;
                if (!resolve_vrt_band(in, vrt, b, bands[b], 0)) {
                    if (verbose) std::printf("Cannot resolve the source of band %d\n", b + 1);
                    return FPL_ERR_OPEN_STACK;
                }
                if (bands[b].bytes != 8) return FPL_ERR_OPEN_STACK;
            }
        }

        // ---- output folder (evd.cpp:226-263) ----
        const std::string outdir = opts->outputFolder;
        struct stat st;
        if (::stat(outdir.c_str(), &st) == 0) {
            if (verbose) std::printf("Output folder : %s already exists \n", outdir.c_str());
            return S_ISDIR(st.st_mode) ? FPL_ERR_OUT_EXISTS_DIR : FPL_ERR_OUT_EXISTS_FILE;
        }
        if (::mkdir(outdir.c_str(), 0777) != 0) return FPL_ERR_OUT_MKDIR;

        // ---- outputs (evd.cpp:266-366) ----
        std::vector<std::unique_ptr<OutFile>> slcs(nbands);
        for (int b = 0; b < nbands; ++b) {
            slcs[b].reset(new OutFile());
            if (!create_output(join_path(outdir, dates[b] + ".slc"), cols, rows, 8, 6, *slcs[b]))
                return FPL_ERR_CREATE_SLC;
        }
        OutFile corr, comp;
        if (!create_output(join_path(outdir, "tcorr.bin"), cols, rows, 4, 4, corr)) return FPL_ERR_CREATE_AUX;
        const std::string cdir = opts->outputCompressedSlcFolder ? opts->outputCompressedSlcFolder : outdir;
        const std::string cname = opts->compSlc ? opts->compSlc : "compslc.bin";
        if (!create_output(join_path(cdir, cname), cols, rows, 8, 6, comp)) return FPL_ERR_CREATE_AUX;

        // ---- block sizes (evd.cpp:169-187) ----
        const int blocksize = opts->blocksize > 0 ? opts->blocksize : 64;
        int boxesperblock = int((opts->memsize * 1.0e6) / cols) / (blocksize * (nbands * 20 + 4 + nulong));
        int blockysize = boxesperblock * blocksize;
        if (blockysize < blocksize) blockysize = blocksize;
        if (blockysize > rows) blockysize = rows;
        if (verbose) std::printf("Block size = %d lines \n", blockysize);

        fpl_ctx *ctx = nullptr;
        int rc = fpl_ctx_create(opts->device, &ctx);
        if (rc) return rc;
        std::unique_ptr<fpl_ctx, int (*)(fpl_ctx *)> guard(ctx, fpl_ctx_destroy);

        std::vector<float> stack((size_t)nbands * blockysize * cols * 2);
        std::vector<uint32_t> nmap((size_t)blockysize * cols * nulong);
        std::vector<float> phase((size_t)nbands * blockysize * cols * 2), tcorr((size_t)blockysize * cols),
            compv((size_t)blockysize * cols * 2);

        int yoff = 0, blockcount = 0;
        while (yoff < rows) {
            blockcount++;
            int inysize = blockysize;
            if (yoff + inysize > rows) inysize = rows - yoff;
            int firstlinetowrite, linestowrite, rollback;       // evd.cpp:419-443
            if (blockcount == 1) {
                firstlinetowrite = 0;
                linestowrite = inysize - Ny;
                rollback = Ny;
                if (yoff + blockysize >= rows) { linestowrite = inysize; rollback = 0; }
            } else if (yoff + blockysize >= rows) {
                firstlinetowrite = Ny;
                linestowrite = inysize - Ny;
                rollback = 0;
            } else {
                firstlinetowrite = Ny;
                linestowrite = inysize - 2 * Ny;
                rollback = 0;
            }
            const size_t plane = (size_t)inysize * cols;
            for (int b = 0; b < nbands; ++b)
                if (!read_rows(bands[b], cols, yoff, inysize, stack.data() + 2 * b * plane)) return FPL_ERR_READ_STACK;
            if (!read_rows(wband[0], cols, yoff, inysize, nmap.data())) return FPL_ERR_READ_WEIGHTS;

            fpl_job job;
            std::memset(&job, 0, sizeof(job));
            job.rows = inysize;
            job.cols = cols;
            job.nbands = nbands;
            job.half_window_y = Ny;
            job.half_window_x = Nx;
            job.method = meth;
            job.semantics = opts->semantics;
            job.mini_stack_count = opts->miniStackCount;
            job.band_width = opts->bandWidth;
            job.min_neighbors = opts->minNeighbors;
            job.precision = opts->precision;
            job.memory = FPL_MEM_HOST;
            job.row_begin = firstlinetowrite;
            job.row_end = firstlinetowrite + linestowrite;
            job.stack = stack.data();
            job.nmap = nmap.data();
            job.phase = phase.data();
            job.tcorr = tcorr.data();
            job.comp = compv.data();
            if (linestowrite > 0) {
                rc = fpl_run(ctx, &job);
                if (rc) return rc;
                const size_t off = (size_t)firstlinetowrite * cols;
                for (int b = 0; b < nbands; ++b)
                    if (!write_rows(*slcs[b], cols, 8, yoff + firstlinetowrite, linestowrite,
                                    phase.data() + 2 * (b * plane + off)))
                        return FPL_ERR_WRITE_SLC;
                if (!write_rows(corr, cols, 4, yoff + firstlinetowrite, linestowrite, tcorr.data() + off))
                    return FPL_ERR_WRITE_AUX;
                if (!write_rows(comp, cols, 8, yoff + firstlinetowrite, linestowrite, compv.data() + 2 * off))
                    return FPL_ERR_WRITE_AUX;
            }
            if (yoff + blockysize < rows) yoff += linestowrite - rollback;   // evd.cpp:861-868
            else yoff = rows;
            if (verbose) std::printf("block %d done (%d/%d lines)\n", blockcount, yoff, rows);
        }
        return FPL_OK;
    });
}

}  // extern "C"
