// vgb_quipu.cpp -- host side of Vira's DEM Quipu files (.qld): the LZ4 block codec, the file
// index and the quantised payload reads that feed the device decode, and the pyramid writer.
//
// Layout restated from include/implementation/quipu/quipu_io.ipp and dem_quipu.ipp:
//   header  "QUIPU" | u16 class id (2002) | transformation: vec3d position, mat3d rotation,
//           vec3d scale (each: u16 class id, u8 N [, u8 M], N(xM) doubles) | u16 LoD count |
//           u8 albedo flag | vec3f normal | f32 cone angle | LoD count x (f64 GSD, u64 offset)
//   LoD     DEMProjection: u32 W, u32 H, f64[2] pixel scale, u32[2] tile definitions, u32 tile
//           row, u32 tile col, f64 xoff, yoff, dx, dy, u8 isOGR [u32 n + n chars, f64[2]
//           row/col rotation, f64[2] model tie point] |
//           heights: f32[2] min/max, u16 precision class, image | [u8 albedo type, payload]
//   image   u16 class id, u32 W, u32 H, u8 compressed, then either u64 raw size, u64 block
//           size, LZ4 block of the row-major pixels, or the raw pixels column by column
//           (x outer, y inner: quipu_io.ipp:733-740).
// Fixed point (image_utils.ipp:485-527): code = T((m - 1) * (v - min) / (max - min) + 1) with
// m = max of T, 0 for +-inf (and NaN, which the reference converts through an undefined cast
// that x86-64 turns into 0); decode v = (max - min) * (code / (m - 1)) + min, +inf for code 0.
// Compiled with -ffp-contract=off: the FP32 expressions round as written.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "../../include/vgb.h"
#include "vgb_internal.h"

namespace {

thread_local std::string g_quipu_err;

vgb_status qfail(const std::string& m, vgb_status s = VGB_ERR_INVALID_ARGUMENT) {
    g_quipu_err = m;
    return s;
}

// ------------------------------------------------------------------ LZ4 block format
// Sequences of: token (literal length << 4 | match length - 4), optional 255-run length bytes,
// literals, 16-bit little-endian offset, optional match length bytes; the last sequence has
// literals only.  Matches are at least 4 bytes and reach back at most 65535 bytes.
constexpr size_t kMinMatch = 4, kLastLiterals = 5, kMatchStartLimit = 12;

int64_t lz4_decode(const uint8_t* src, size_t n, uint8_t* dst, size_t cap) {
    if (n == 0) return -1;
    size_t ip = 0, op = 0;
    for (;;) {
        const unsigned token = src[ip++];
        size_t lit = token >> 4;
        if (lit == 15) {
            unsigned b;
            do {
                if (ip >= n) return -1;
                b = src[ip++];
                lit += b;
            } while (b == 255);
        }
        if (lit > n - ip || lit > cap - op) return -1;
        std::memcpy(dst + op, src + ip, lit);
        ip += lit;
        op += lit;
        if (ip == n) return (int64_t)op;  // the last sequence ends with its literals
        if (n - ip < 2) return -1;
        const size_t off = (size_t)src[ip] | ((size_t)src[ip + 1] << 8);
        ip += 2;
        if (off == 0 || off > op) return -1;
        size_t ml = token & 15u;
        if (ml == 15) {
            unsigned b;
            do {
                if (ip >= n) return -1;
                b = src[ip++];
                ml += b;
            } while (b == 255);
        }
        ml += kMinMatch;
        if (ml > cap - op) return -1;
        uint8_t* d = dst + op;
        if (off >= ml) {
            std::memcpy(d, d - off, ml);
        } else {
            // overlapping: the match repeats with period `off`, so any multiple of it is a
            // period too -- copy in non-overlapping chunks whose distance doubles
            size_t rem = ml, dist = off;
            while (rem) {
                const size_t c = std::min(dist, rem);
                std::memcpy(d, d - dist, c);
                d += c;
                rem -= c;
                dist *= 2;
            }
        }
        op += ml;
        if (ip >= n) return -1;  // a match must be followed by another sequence
    }
}

uint64_t lz4_bound(uint64_t n) { return n + n / 255 + 16; }

inline uint32_t load32(const uint8_t* p) { uint32_t v; std::memcpy(&v, p, 4); return v; }

void put_length(uint8_t*& op, size_t v) {  // the part of a length beyond 15, as 255-runs
    while (v >= 255) { *op++ = 255; v -= 255; }
    *op++ = (uint8_t)v;
}

// Greedy single-probe matcher (a hash table of the last position of every 4-byte sequence),
// skipping faster through incompressible stretches.  Output obeys the block rules: the last
// 5 bytes are literals and no match starts within the last 12 bytes.
uint64_t lz4_encode(const uint8_t* src, size_t n, uint8_t* dst, uint64_t cap) {
    if (cap < lz4_bound(n)) return 0;
    uint8_t* op = dst;
    size_t anchor = 0;
    auto emit = [&](size_t lit_end, size_t off, size_t ml) {
        const size_t lit = lit_end - anchor;
        uint8_t* token = op++;
        const unsigned lt = lit >= 15 ? 15u : (unsigned)lit;
        if (lit >= 15) put_length(op, lit - 15);
        std::memcpy(op, src + anchor, lit);
        op += lit;
        if (ml == 0) { *token = (uint8_t)(lt << 4); return; }
        *op++ = (uint8_t)(off & 0xFF);
        *op++ = (uint8_t)(off >> 8);
        const size_t mc = ml - kMinMatch;
        *token = (uint8_t)((lt << 4) | (mc >= 15 ? 15u : (unsigned)mc));
        if (mc >= 15) put_length(op, mc - 15);
    };
    if (n > kMatchStartLimit) {
        constexpr int kHashBits = 16;
        std::vector<uint32_t> table((size_t)1 << kHashBits, 0u);   // position + 1, 0 = empty
        const size_t last_start = n - kMatchStartLimit;            // matches start at <= this
        size_t ip = 0;
        while (ip <= last_start) {
            const uint32_t seq = load32(src + ip);
            const uint32_t h = (seq * 2654435761u) >> (32 - kHashBits);
            const uint32_t cand1 = table[h];
            table[h] = (uint32_t)(ip + 1);
            if (cand1 != 0) {
                const size_t cand = cand1 - 1;
                if (ip - cand <= 65535 && load32(src + cand) == seq) {
                    size_t ml = kMinMatch;
                    const size_t max_ml = (n - kLastLiterals) - ip;
                    while (ml < max_ml && src[cand + ml] == src[ip + ml]) ++ml;
                    emit(ip, ip - cand, ml);
                    ip += ml;
                    anchor = ip;
                    continue;
                }
            }
            ip += 1 + ((ip - anchor) >> 6);
        }
    }
    emit(n, 0, 0);
    return (uint64_t)(op - dst);
}

// ------------------------------------------------------------------ file reading
struct File {
    FILE* f = nullptr;
    std::string path;
    bool ok = true;
    ~File() { if (f) std::fclose(f); }
    bool seek(uint64_t pos) { ok = ok && fseeko(f, (off_t)pos, SEEK_SET) == 0; return ok; }
    uint64_t tell() { return (uint64_t)ftello(f); }
    bool read(void* p, size_t n) { ok = ok && std::fread(p, 1, n, f) == n; return ok; }
    template <typename T> T get() { T v{}; read(&v, sizeof(T)); return v; }
    bool skip(uint64_t n) { ok = ok && fseeko(f, (off_t)n, SEEK_CUR) == 0; return ok; }
    uint64_t size() {
        const off_t here = ftello(f);
        fseeko(f, 0, SEEK_END);
        const uint64_t n = (uint64_t)ftello(f);
        fseeko(f, here, SEEK_SET);
        return n;
    }
};

enum : uint16_t { kFloat = 1, kDouble = 2, kU8 = 3, kU16 = 4, kDemPyramid = 2002 };

size_t class_bytes(uint16_t c) { return c == kU8 ? 1 : c == kU16 ? 2 : c == kFloat ? 4 : 0; }

struct ImageRef {              // where an image's pixels sit in the file
    uint16_t cls = 0;
    uint32_t w = 0, h = 0;
    bool compressed = false;
    uint64_t raw_bytes = 0;    // W * H * sizeof(T) (compressed: as stored)
    uint64_t pos = 0;          // first byte of the LZ4 block or of the raw pixels
    uint64_t stored = 0;       // bytes in the file
};

struct Plane { float mn = 0, mx = 0; ImageRef img; };

struct Lod {
    double gsd = 0;
    uint64_t offset = 0;
    vgb_quipu_projection proj{};
    float hmin = 0, hmax = 0;
    uint16_t precision = 0;
    ImageRef heights;
    uint32_t albedo_type = VGB_QUIPU_NO_ALBEDO;
    uint64_t constant_pos = 0;  // constant albedo: nbands floats of the reading program
    std::vector<Plane> planes;  // grey: 1, per band: channels
};

bool read_image_ref(File& f, ImageRef& r) {
    r.cls = f.get<uint16_t>();
    r.w = f.get<uint32_t>();
    r.h = f.get<uint32_t>();
    r.compressed = f.get<uint8_t>() != 0;
    const size_t tb = class_bytes(r.cls);
    if (!f.ok || tb == 0) return false;
    if (r.compressed) {
        r.raw_bytes = f.get<uint64_t>();
        r.stored = f.get<uint64_t>();
        r.pos = f.tell();
        if (r.raw_bytes != (uint64_t)r.w * r.h * tb) return false;
    } else {
        r.raw_bytes = (uint64_t)r.w * r.h * tb;
        r.stored = r.raw_bytes;
        r.pos = f.tell();
    }
    // the pixels must lie inside the file
    if (!f.ok || r.stored > f.size() || r.pos > f.size() - r.stored) return false;
    // an LZ4 block expands at most 255-fold (a match costs at least one byte per 255 output
    // bytes), so a larger claimed size is malformed -- and is never allocated
    if (r.compressed && r.raw_bytes > 255 * r.stored + 255) return false;
    return f.skip(r.stored);
}

}  // namespace

struct vgb_quipu_dem {
    std::string path;
    vgb_quipu_header header{};
    std::vector<Lod> lods;
};

namespace vgb {

// Decodes an image's pixels, row-major, into `out` (raw_bytes bytes).
vgb_status quipu_read_pixels(const std::string& path, const ImageRefView& v, void* out) {
    File f;
    f.f = std::fopen(path.c_str(), "rb");
    if (!f.f) return qfail("cannot open " + path);
    if (!f.seek(v.pos)) return qfail(path + ": truncated");
    if (v.compressed) {
        std::vector<uint8_t> block(v.stored);
        if (!f.read(block.data(), block.size())) return qfail(path + ": truncated LZ4 block");
        const int64_t got = lz4_decode(block.data(), block.size(), (uint8_t*)out, v.raw_bytes);
        if (got != (int64_t)v.raw_bytes) return qfail(path + ": malformed LZ4 block");
        return VGB_OK;
    }
    // raw pixels are stored column by column
    std::vector<uint8_t> col(v.raw_bytes);
    if (!f.read(col.data(), col.size())) return qfail(path + ": truncated image");
    const size_t tb = v.elem, W = v.w, H = v.h;
    uint8_t* o = (uint8_t*)out;
    for (size_t i = 0; i < W; ++i)
        for (size_t j = 0; j < H; ++j) std::memcpy(o + (j * W + i) * tb, col.data() + (i * H + j) * tb, tb);
    return VGB_OK;
}

vgb_status quipu_lod_payload(const vgb_quipu_dem* q, uint32_t lod, QuipuPayload* out) {
    if (!q || lod >= q->lods.size()) return qfail("quipu: LoD index out of range");
    const Lod& L = q->lods[lod];
    auto view = [](const ImageRef& r) {
        return ImageRefView{r.pos, r.stored, r.raw_bytes, r.w, r.h, (uint32_t)class_bytes(r.cls), r.compressed};
    };
    out->path = q->path;
    out->heights = view(L.heights);
    out->precision = L.precision;
    out->hmin = L.hmin;
    out->hmax = L.hmax;
    out->albedo_type = L.albedo_type;
    out->constant_pos = L.constant_pos;
    out->planes.clear();
    for (const Plane& p : L.planes) out->planes.push_back(QuipuPlane{p.mn, p.mx, view(p.img)});
    out->proj = L.proj;
    return VGB_OK;
}

vgb_status quipu_read_constant(const std::string& path, uint64_t pos, uint32_t nbands, float* out) {
    File f;
    f.f = std::fopen(path.c_str(), "rb");
    if (!f.f) return qfail("cannot open " + path);
    if (!f.seek(pos) || !f.read(out, sizeof(float) * nbands)) return qfail(path + ": truncated constant albedo");
    return VGB_OK;
}

void quipu_set_error(const std::string& m) { g_quipu_err = m; }

}  // namespace vgb

extern "C" {

VGB_API const char* vgb_quipu_last_error(void) { return g_quipu_err.c_str(); }

VGB_API int64_t vgb_lz4_decompress(const void* src, uint64_t src_size, void* dst, uint64_t dst_cap) {
    if (!src || (!dst && dst_cap)) return -1;
    return lz4_decode((const uint8_t*)src, (size_t)src_size, (uint8_t*)dst, (size_t)dst_cap);
}

VGB_API uint64_t vgb_lz4_bound(uint64_t n) { return lz4_bound(n); }

VGB_API uint64_t vgb_lz4_compress(const void* src, uint64_t n, void* dst, uint64_t dst_cap) try {
    if ((!src && n) || !dst) return 0;
    return lz4_encode((const uint8_t*)src, (size_t)n, (uint8_t*)dst, dst_cap);
} catch (...) {
    vgb::status_of_exception(&g_quipu_err);
    return 0;  // the encoder's hash table could not be allocated
}

// DEMQuipu::DEMQuipu (dem_quipu.ipp:29-60), quipu::open (quipu_io.ipp:24-54), and an index of
// the LoD blocks (readDEMProjection :573-590, readDEMHeights :601-626, readAlbedos_f :643-653,
// readAlbedos :672-702, readImage :717-752).
VGB_API vgb_status vgb_quipu_open(const char* path, vgb_quipu_dem** out) try {
    if (!path || !out) return qfail("quipu_open: null argument");
    *out = nullptr;
    File f;
    f.path = path;
    f.f = std::fopen(path, "rb");
    if (!f.f) return qfail(std::string("There is no file with path: ") + path);
    char ident[5];
    if (!f.read(ident, 5) || std::memcmp(ident, "QUIPU", 5) != 0)
        return qfail(std::string(path) + " exists, but is not a valid Quipu!");
    auto q = std::make_unique<vgb_quipu_dem>();
    q->path = path;
    vgb_quipu_header& hd = q->header;
    hd.class_id = f.get<uint16_t>();
    if (f.ok && hd.class_id != kDemPyramid) return qfail(std::string(path) + ": not a DEM pyramid Quipu");
    auto vec = [&](double* v, int n) {
        const uint16_t c = f.get<uint16_t>();
        const uint8_t k = f.get<uint8_t>();
        if (!f.ok || k != n || (c != kDouble && c != kFloat)) { f.ok = false; return; }
        for (int i = 0; i < n; ++i) v[i] = c == kDouble ? f.get<double>() : (double)f.get<float>();
    };
    vec(hd.position, 3);
    {
        const uint16_t c = f.get<uint16_t>();
        const uint8_t n = f.get<uint8_t>(), m = f.get<uint8_t>();
        if (!f.ok || n != 3 || m != 3 || (c != kDouble && c != kFloat)) return qfail(std::string(path) + ": bad rotation");
        for (int i = 0; i < 9; ++i) hd.rotation[i] = c == kDouble ? f.get<double>() : (double)f.get<float>();
    }
    vec(hd.scale, 3);
    hd.num_lods = f.get<uint16_t>();
    hd.has_albedos = f.get<uint8_t>() != 0 ? 1u : 0u;
    {
        const uint16_t c = f.get<uint16_t>();
        const uint8_t k = f.get<uint8_t>();
        if (!f.ok || k != 3 || c != kFloat) return qfail(std::string(path) + ": bad normal");
        for (int i = 0; i < 3; ++i) hd.normal[i] = f.get<float>();
    }
    hd.cone_angle = f.get<float>();
    if (!f.ok) return qfail(std::string(path) + ": truncated header");
    if (hd.num_lods == 0 || hd.num_lods > VGB_QUIPU_MAX_LODS)
        return qfail(std::string(path) + ": LoD count outside 1.." + std::to_string(VGB_QUIPU_MAX_LODS));
    q->lods.resize(hd.num_lods);
    for (Lod& L : q->lods) {
        L.gsd = f.get<double>();
        L.offset = f.get<uint64_t>();
    }
    if (!f.ok) return qfail(std::string(path) + ": truncated table of contents");
    for (size_t i = 0; i < q->lods.size(); ++i) {
        Lod& L = q->lods[i];
        const std::string where = std::string(path) + ": LoD " + std::to_string(i);
        if (!f.seek(L.offset)) return qfail(where + ": offset beyond the file");
        vgb_quipu_projection& p = L.proj;
        p.width = f.get<uint32_t>(); p.height = f.get<uint32_t>();
        p.pixel_scale[0] = f.get<double>(); p.pixel_scale[1] = f.get<double>();
        p.tile_definitions[0] = f.get<uint32_t>(); p.tile_definitions[1] = f.get<uint32_t>();
        p.tile_row = f.get<uint32_t>(); p.tile_col = f.get<uint32_t>();
        p.xoff = f.get<double>(); p.yoff = f.get<double>(); p.dx = f.get<double>(); p.dy = f.get<double>();
        p.is_ogr = f.get<uint8_t>() != 0 ? 1u : 0u;
        if (p.is_ogr) {
            const uint32_t len = f.get<uint32_t>();
            if (!f.skip(len)) return qfail(where + ": truncated projection string");
            p.row_col_rotation[0] = f.get<double>(); p.row_col_rotation[1] = f.get<double>();
            p.model_tie_point[0] = f.get<double>(); p.model_tie_point[1] = f.get<double>();
        }
        L.hmin = f.get<float>();
        L.hmax = f.get<float>();
        L.precision = f.get<uint16_t>();
        if (!f.ok) return qfail(where + ": truncated");
        if (L.precision != kU8 && L.precision != kU16 && L.precision != kFloat)
            return qfail(where + ": height precision class " + std::to_string(L.precision) + " is not uint8/uint16/float");
        if (!read_image_ref(f, L.heights) || L.heights.cls != L.precision)
            return qfail(where + ": bad or truncated height image");
        if (hd.has_albedos) {
            L.albedo_type = f.get<uint8_t>();
            if (!f.ok) return qfail(where + ": truncated albedo");
            if (L.albedo_type == 0) {
                L.constant_pos = f.tell();
            } else if (L.albedo_type == 1) {
                Plane pl;
                pl.mn = f.get<float>(); pl.mx = f.get<float>();
                if (!read_image_ref(f, pl.img) || pl.img.cls != kU8) return qfail(where + ": bad albedo image");
                L.planes.push_back(pl);
            } else if (L.albedo_type == 2) {
                const uint32_t nch = f.get<uint32_t>();
                f.get<uint8_t>();  // compressed flag of the channel set (each image repeats it)
                if (!f.ok || nch == 0 || nch > 64) return qfail(where + ": bad albedo channel count");
                for (uint32_t c = 0; c < nch; ++c) {
                    Plane pl;
                    pl.mn = f.get<float>(); pl.mx = f.get<float>();
                    if (!read_image_ref(f, pl.img) || pl.img.cls != kU8) return qfail(where + ": bad albedo image");
                    L.planes.push_back(pl);
                }
            } else {
                return qfail(where + ": unknown albedo type " + std::to_string(L.albedo_type));
            }
            for (const Plane& pl : L.planes)
                if (pl.img.w != L.heights.w || pl.img.h != L.heights.h)
                    return qfail(where + ": albedo and heights differ in resolution");
        }
    }
    *out = q.release();
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(&g_quipu_err);
}

VGB_API void vgb_quipu_close(vgb_quipu_dem* q) { delete q; }

VGB_API vgb_status vgb_quipu_get_header(const vgb_quipu_dem* q, vgb_quipu_header* out) try {
    if (!q || !out) return qfail("quipu_get_header: null argument");
    *out = q->header;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(&g_quipu_err);
}

VGB_API vgb_status vgb_quipu_get_lod(const vgb_quipu_dem* q, uint32_t lod, vgb_quipu_lod_info* out) try {
    if (!q || !out) return qfail("quipu_get_lod: null argument");
    if (lod >= q->lods.size()) return qfail("quipu_get_lod: LoD index out of range");
    const Lod& L = q->lods[lod];
    vgb_quipu_lod_info i{};
    i.gsd = L.gsd;
    i.offset = L.offset;
    i.width = L.heights.w;
    i.height = L.heights.h;
    i.projection = L.proj;
    i.height_min = L.hmin;
    i.height_max = L.hmax;
    i.precision = L.precision;
    i.compressed = L.heights.compressed ? 1u : 0u;
    i.albedo_type = L.albedo_type;
    i.albedo_channels = L.albedo_type == 2 ? (uint32_t)L.planes.size() : (L.albedo_type == 1 ? 1u : 0u);
    *out = i;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(&g_quipu_err);
}

VGB_API uint32_t vgb_quipu_select_lod(const vgb_quipu_dem* q, double required_gsd) {
    if (!q || q->lods.empty()) return 0;
    uint32_t sel = 0;
    for (uint32_t i = 1; i < q->lods.size(); ++i) {
        if (q->lods[i].gsd <= required_gsd) sel = i;
        else break;
    }
    return sel;
}

VGB_API vgb_status vgb_quipu_read_heights(vgb_quipu_dem* q, uint32_t lod, float* heights) try {
    if (!q || !heights) return qfail("quipu_read_heights: null argument");
    vgb::QuipuPayload pl;
    vgb_status s = vgb::quipu_lod_payload(q, lod, &pl);
    if (s != VGB_OK) return s;
    const size_t n = (size_t)pl.heights.w * pl.heights.h;
    std::vector<uint8_t> raw(pl.heights.raw_bytes);
    if ((s = vgb::quipu_read_pixels(pl.path, pl.heights, raw.data())) != VGB_OK) return s;
    const float mn = pl.hmin, mx = pl.hmax;
    if (pl.precision == kFloat) {
        std::memcpy(heights, raw.data(), n * sizeof(float));
    } else if (pl.precision == kU8) {
        for (size_t k = 0; k < n; ++k) heights[k] = vgb::quipu_dequantize(raw[k], 255.f, mn, mx);
    } else {
        const uint16_t* r = (const uint16_t*)raw.data();
        for (size_t k = 0; k < n; ++k) heights[k] = vgb::quipu_dequantize(r[k], 65535.f, mn, mx);
    }
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(&g_quipu_err);
}

VGB_API vgb_status vgb_quipu_read_albedo(vgb_quipu_dem* q, uint32_t lod, uint32_t nbands, float* albedo) try {
    if (!q || !albedo) return qfail("quipu_read_albedo: null argument");
    vgb::QuipuPayload pl;
    vgb_status s = vgb::quipu_lod_payload(q, lod, &pl);
    if (s != VGB_OK) return s;
    if (pl.albedo_type == VGB_QUIPU_NO_ALBEDO) return qfail("quipu_read_albedo: the file stores no albedo", VGB_ERR_NOT_READY);
    if (pl.albedo_type == 0) {
        if (nbands == 0 || nbands > VGB_MAX_BANDS) return qfail("quipu_read_albedo: nbands must be 1..8");
        return vgb::quipu_read_constant(pl.path, pl.constant_pos, nbands, albedo);
    }
    if (pl.albedo_type == 2 && pl.planes.size() != nbands)
        return qfail("Quipu file uses a Spectral albedo with " + std::to_string(pl.planes.size()) +
                     " channels, while the reader has " + std::to_string(nbands) + " bands");
    const size_t n = (size_t)pl.heights.w * pl.heights.h, nc = pl.planes.size();
    std::vector<uint8_t> codes(n);
    for (size_t c = 0; c < nc; ++c) {
        if ((s = vgb::quipu_read_pixels(pl.path, pl.planes[c].img, codes.data())) != VGB_OK) return s;
        for (size_t k = 0; k < n; ++k)
            albedo[k * nc + c] = vgb::quipu_dequantize(codes[k], 255.f, pl.planes[c].mn, pl.planes[c].mx);
    }
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(&g_quipu_err);
}

}  // extern "C"

// ------------------------------------------------------------------ writer
namespace {

struct Writer {
    std::vector<uint8_t> buf;
    template <typename T> void put(T v) {
        const size_t o = buf.size();
        buf.resize(o + sizeof(T));
        std::memcpy(buf.data() + o, &v, sizeof(T));
    }
    void bytes(const void* p, size_t n) {
        const size_t o = buf.size();
        buf.resize(o + n);
        if (n) std::memcpy(buf.data() + o, p, n);
    }
};

// Image<float>::min / max (image.ipp:693-730): over the finite, non-NaN values, starting from
// FLT_MAX / lowest.
void valid_minmax(const float* v, size_t n, size_t stride, float& mn, float& mx) {
    mn = std::numeric_limits<float>::max();
    mx = std::numeric_limits<float>::lowest();
    for (size_t k = 0; k < n; ++k) {
        const float x = v[k * stride];
        if (std::isinf(x) || std::isnan(x)) continue;
        if (mn > x) mn = x;
        if (mx < x) mx = x;
    }
}

template <typename T>
T to_fixed(float value, float mn, float mx) {
    if (std::isinf(value)) return 0;
    const float m = (float)std::numeric_limits<T>::max();
    const float v = (value - mn) / (mx - mn);
    const float code = ((m - 1.f) * v) + 1.f;
    if (std::isnan(code)) return 0;  // undefined cast in the reference; x86-64 yields 0
    return (T)code;
}

// writeImage (quipu_io.ipp:706-731): row-major LZ4 block, or raw pixels column by column.
template <typename T>
bool write_image(Writer& w, uint16_t cls, const T* px, uint32_t W, uint32_t H, bool compress) {
    w.put<uint16_t>(cls);
    w.put<uint32_t>(W);
    w.put<uint32_t>(H);
    w.put<uint8_t>(compress ? 1 : 0);
    const size_t raw = (size_t)W * H * sizeof(T);
    if (compress) {
        if (raw > 0x7E000000ull) return false;  // LZ4's input limit, which the reference hits too
        w.put<uint64_t>(raw);
        std::vector<uint8_t> blk(lz4_bound(raw));
        const uint64_t cs = lz4_encode((const uint8_t*)px, raw, blk.data(), blk.size());
        if (cs == 0) return false;
        w.put<uint64_t>(cs);
        w.bytes(blk.data(), cs);
    } else {
        const size_t o = w.buf.size();
        w.buf.resize(o + raw);
        uint8_t* d = w.buf.data() + o;
        for (size_t i = 0; i < W; ++i)
            for (size_t j = 0; j < H; ++j) std::memcpy(d + (i * H + j) * sizeof(T), px + j * W + i, sizeof(T));
    }
    return true;
}

template <typename T>
bool write_fixed(Writer& w, uint16_t cls, const float* v, size_t stride, uint32_t W, uint32_t H, float mn, float mx,
                 bool compress) {
    std::vector<T> q((size_t)W * H);
    for (size_t k = 0; k < q.size(); ++k) q[k] = to_fixed<T>(v[k * stride], mn, mx);
    return write_image(w, cls, q.data(), W, H, compress);
}

void put_projection(Writer& w, const vgb_quipu_projection& p) {
    w.put<uint32_t>(p.width); w.put<uint32_t>(p.height);
    w.put<double>(p.pixel_scale[0]); w.put<double>(p.pixel_scale[1]);
    w.put<uint32_t>(p.tile_definitions[0]); w.put<uint32_t>(p.tile_definitions[1]);
    w.put<uint32_t>(p.tile_row); w.put<uint32_t>(p.tile_col);
    w.put<double>(p.xoff); w.put<double>(p.yoff); w.put<double>(p.dx); w.put<double>(p.dy);
    w.put<uint8_t>(0);  // isOGR: map projections are not written (they need GDAL)
}

}  // namespace

extern "C" VGB_API vgb_status vgb_quipu_write(const char* path, const vgb_quipu_lod_data* lods, uint32_t nlods,
                                             const double position[3], const double rotation[9],
                                             const double scale[3], int write_albedos, int compress) try {
    if (!path || !lods || !position || !rotation || !scale) return qfail("quipu_write: null argument");
    if (nlods == 0 || nlods > VGB_QUIPU_MAX_LODS)
        return qfail("quipu_write: LoD count outside 1.." + std::to_string(VGB_QUIPU_MAX_LODS));
    const uint32_t atype = lods[0].albedo_type;
    for (uint32_t i = 0; i < nlods; ++i) {
        const vgb_quipu_lod_data& L = lods[i];
        if (!L.heights || L.projection.width < 2 || L.projection.height < 2)
            return qfail("quipu_write: LoD " + std::to_string(i) + " has no heights or fewer than 2x2 posts");
        if (L.projection.is_ogr) return qfail("quipu_write: map-projected (OGR) LoDs need GDAL, which is absent");
        if (write_albedos) {
            if (L.albedo_type != atype) return qfail("quipu_write: every LoD must carry the base LoD's albedo type");
            if (atype > 2 || !L.albedo) return qfail("quipu_write: albedo type outside 0..2 or null albedo");
            if ((atype != 1) && (L.nbands == 0 || L.nbands > VGB_MAX_BANDS))
                return qfail("quipu_write: albedo bands outside 1..8");
        }
    }
    Writer w;
    w.bytes("QUIPU", 5);
    w.put<uint16_t>(kDemPyramid);
    auto vec3d = [&](const double* v) { w.put<uint16_t>(kDouble); w.put<uint8_t>(3); for (int i = 0; i < 3; ++i) w.put<double>(v[i]); };
    vec3d(position);
    w.put<uint16_t>(kDouble); w.put<uint8_t>(3); w.put<uint8_t>(3);
    for (int i = 0; i < 9; ++i) w.put<double>(rotation[i]);
    vec3d(scale);
    w.put<uint16_t>((uint16_t)nlods);
    w.put<uint8_t>(write_albedos ? 1 : 0);

    // normal cone of the coarsest LoD's mesh (dem_quipu.ipp:256-270)
    {
        const vgb_quipu_lod_data& S = lods[nlods - 1];
        const uint32_t W = S.projection.width, H = S.projection.height;
        const size_t nv = (size_t)W * H;
        std::vector<float> pos(3 * nv), nrm(3 * nv);
        std::vector<uint32_t> idx(6 * (size_t)(W - 1) * (H - 1));
        uint32_t nt = 0;
        vgb::DemPose pose = vgb::dem_pose(S.projection);
        vgb::dem_vertices_host(S.heights, W, H, pose, pos.data());
        vgb::dem_faces_host(S.heights, W, H, idx.data(), &nt);
        vgb_status s = vgb_compute_vertex_normals(pos.data(), (uint32_t)nv, idx.data(), nt, nrm.data());
        if (s != VGB_OK) return qfail("quipu_write: normals of the coarsest LoD failed");
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (size_t v = 0; v < nv; ++v) { sx += nrm[3 * v]; sy += nrm[3 * v + 1]; sz += nrm[3 * v + 2]; }
        const float inv = 1.0f / std::sqrt((sx * sx + sy * sy) + sz * sz);
        const float n0 = sx * inv, n1 = sy * inv, n2 = sz * inv;
        float cone = 0.f;
        for (size_t v = 0; v < nv; ++v) {
            const float d = (nrm[3 * v] * n0 + nrm[3 * v + 1] * n1) + nrm[3 * v + 2] * n2;
            const float a = std::acos(d);
            cone = (cone < a) ? a : cone;  // std::max(cone, a)
        }
        w.put<uint16_t>(kFloat); w.put<uint8_t>(3);
        w.put<float>(n0); w.put<float>(n1); w.put<float>(n2);
        w.put<float>(cone);
    }
    const size_t header = w.buf.size();
    const size_t toc = header;
    w.buf.resize(header + 16 * (size_t)nlods, 0);

    float hmn, hmx;
    valid_minmax(lods[0].heights, (size_t)lods[0].projection.width * lods[0].projection.height, 1, hmn, hmx);
    std::vector<uint64_t> offsets(nlods);
    for (uint32_t i = 0; i < nlods; ++i) {
        const vgb_quipu_lod_data& L = lods[i];
        const uint32_t W = L.projection.width, H = L.projection.height;
        offsets[i] = w.buf.size();
        put_projection(w, L.projection);
        // writeDEMHeights (quipu_io.ipp:575-599)
        const float gsd = (float)std::min(L.projection.dx * L.projection.pixel_scale[0],
                                          L.projection.dy * L.projection.pixel_scale[1]);
        const float gsd_scale = gsd / 50.f;
        const float delta = hmx - hmn;
        w.put<float>(hmn);
        w.put<float>(hmx);
        bool ok;
        if (delta / 255.f < gsd_scale) {
            w.put<uint16_t>(kU8);
            ok = write_fixed<uint8_t>(w, kU8, L.heights, 1, W, H, hmn, hmx, compress != 0);
        } else if (delta / 65535.f < gsd_scale) {
            w.put<uint16_t>(kU16);
            ok = write_fixed<uint16_t>(w, kU16, L.heights, 1, W, H, hmn, hmx, compress != 0);
        } else {
            w.put<uint16_t>(kFloat);
            ok = write_image(w, kFloat, L.heights, W, H, compress != 0);
        }
        if (!ok) return qfail("quipu_write: LoD " + std::to_string(i) + " is too large for one LZ4 block");
        if (write_albedos) {
            w.put<uint8_t>((uint8_t)atype);
            const size_t n = (size_t)W * H;
            if (atype == 0) {
                for (uint32_t b = 0; b < L.nbands; ++b) w.put<float>(L.albedo[b]);
            } else if (atype == 1) {
                float mn, mx;
                valid_minmax(L.albedo, n, 1, mn, mx);
                w.put<float>(mn); w.put<float>(mx);
                ok = write_fixed<uint8_t>(w, kU8, L.albedo, 1, W, H, mn, mx, compress != 0);
            } else {
                w.put<uint32_t>(L.nbands);
                w.put<uint8_t>(compress ? 1 : 0);
                for (uint32_t b = 0; b < L.nbands && ok; ++b) {
                    float mn, mx;
                    valid_minmax(L.albedo + b, n, L.nbands, mn, mx);
                    w.put<float>(mn); w.put<float>(mx);
                    ok = write_fixed<uint8_t>(w, kU8, L.albedo + b, L.nbands, W, H, mn, mx, compress != 0);
                }
            }
            if (!ok) return qfail("quipu_write: albedo of LoD " + std::to_string(i) + " is too large for one LZ4 block");
        }
    }
    for (uint32_t i = 0; i < nlods; ++i) {
        const double g = lods[i].projection.dx * lods[i].projection.pixel_scale[0];
        std::memcpy(w.buf.data() + toc + 16 * (size_t)i, &g, 8);
        std::memcpy(w.buf.data() + toc + 16 * (size_t)i + 8, &offsets[i], 8);
    }
    // DEMQuipu::write forces the .qld extension and creates the parent folders (dem_quipu.ipp:227-229)
    std::filesystem::path fp(path);
    fp.replace_extension(".qld");
    std::error_code ec;
    if (fp.has_parent_path()) std::filesystem::create_directories(fp.parent_path(), ec);
    FILE* f = std::fopen(fp.string().c_str(), "wb");
    if (!f) return qfail("quipu_write: cannot create " + fp.string());
    const bool good = std::fwrite(w.buf.data(), 1, w.buf.size(), f) == w.buf.size();
    if (std::fclose(f) != 0 || !good) return qfail("quipu_write: write failed for " + fp.string());
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(&g_quipu_err);
}
