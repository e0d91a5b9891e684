// .holo files: reading and writing the reference's recording format, and conversion of older
// footers and compute-settings documents to the current version.
//
// Reference behaviour (Holovibes):
//   layout       Backend/includes/io/holo_file.hh:1-81: a 64-byte header (packed on 2 bytes:
//                "HOLO", version u16, bits per pixel u16, width u32, height u32, image count u32,
//                data size u64, endianness u8, data type u8, 34 bytes of padding), the raw frames,
//                then a JSON footer {"compute_settings": {...}, "info": {...}}; version 7
//   reader       Backend/sources/io/input_file/input_holo_file.cc:18-157 (magic and data-size
//                checks, footer = the bytes after the frames, pixel size from
//                info.pixel_pitch.x, camera_fps defaulting to input_fps)
//   writer       Backend/sources/io/output_file/output_holo_file.cc:10-131 (bits = depth * 8,
//                little endian, the image count and data size corrected when the file is closed)
//   versions     Backend/sources/version/holo_file_converter.cc:7-121 (footers of versions 2..6
//                patched forward; 5 and 6 share the current footer layout, 7 only added the data
//                type to the header) and compute_settings_converter.cc (v0 -> v1)
// The header is serialised field by field in little-endian order, not through a packed struct.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "hv_internal.h"
#include "json_lite.h"
#include "settings_internal.h"

using namespace hv;

struct hv_holo_file
{
    FILE* f = nullptr;
    hv_holo_header hdr{};
    uint64_t frame_bytes = 0;
    json::Value footer;  // converted to the current layout (empty object when the file has none)
    bool has_footer = false;
};

struct hv_holo_writer
{
    FILE* f = nullptr;
    hv_holo_header hdr{};
    uint64_t frame_bytes = 0;
    uint64_t frames = 0;
};

namespace {

constexpr uint16_t kHoloVersion = 7;
constexpr size_t kHeaderBytes = 64;

void put16(uint8_t* p, uint16_t v)
{
    p[0] = static_cast<uint8_t>(v);
    p[1] = static_cast<uint8_t>(v >> 8);
}
void put32(uint8_t* p, uint32_t v)
{
    for (int i = 0; i < 4; ++i)
        p[i] = static_cast<uint8_t>(v >> (8 * i));
}
void put64(uint8_t* p, uint64_t v)
{
    for (int i = 0; i < 8; ++i)
        p[i] = static_cast<uint8_t>(v >> (8 * i));
}
uint16_t get16(const uint8_t* p) { return static_cast<uint16_t>(p[0] | (p[1] << 8)); }
uint32_t get32(const uint8_t* p)
{
    uint32_t v = 0;
    for (int i = 3; i >= 0; --i)
        v = (v << 8) | p[i];
    return v;
}
uint64_t get64(const uint8_t* p)
{
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i)
        v = (v << 8) | p[i];
    return v;
}

void encode_header(const hv_holo_header& h, uint8_t out[kHeaderBytes])
{
    std::memset(out, 0, kHeaderBytes);
    std::memcpy(out, h.magic, 4);
    put16(out + 4, h.version);
    put16(out + 6, h.bits_per_pixel);
    put32(out + 8, h.width);
    put32(out + 12, h.height);
    put32(out + 16, h.img_nb);
    put64(out + 20, h.total_data_size);
    out[28] = h.endianness;
    out[29] = h.data_type;
}

void decode_header(const uint8_t in[kHeaderBytes], hv_holo_header& h)
{
    std::memcpy(h.magic, in, 4);
    h.version = get16(in + 4);
    h.bits_per_pixel = get16(in + 6);
    h.width = get32(in + 8);
    h.height = get32(in + 12);
    h.img_nb = get32(in + 16);
    h.total_data_size = get64(in + 20);
    h.endianness = in[28];
    h.data_type = h.version >= 7 ? in[29] : 0;  // versions before 7 are raw recordings
}

bool seek(FILE* f, uint64_t off) { return fseeko(f, static_cast<off_t>(off), SEEK_SET) == 0; }

json::Value obj()
{
    json::Value v;
    v.kind = json::Value::Object;
    return v;
}
json::Value num(double x)
{
    json::Value v;
    v.kind = json::Value::Number;
    v.num = x;
    return v;
}
json::Value str(const std::string& s)
{
    json::Value v;
    v.kind = json::Value::String;
    v.str = s;
    return v;
}

json::Value* child(json::Value& v, const std::string& k)
{
    return v.kind == json::Value::Object ? v.find(k) : nullptr;
}

// Sets v[k] (object v), replacing an existing entry.
void put(json::Value& v, const std::string& k, json::Value x)
{
    if (json::Value* c = child(v, k))
        *c = std::move(x);
    else
        v.obj.emplace_back(k, std::move(x));
}

// Removes and returns v[k] (null when absent).
json::Value take(json::Value& v, const std::string& k)
{
    if (v.kind != json::Value::Object)
        return json::Value{};
    for (size_t i = 0; i < v.obj.size(); ++i)
        if (v.obj[i].first == k)
        {
            json::Value x = std::move(v.obj[i].second);
            v.obj.erase(v.obj.begin() + static_cast<std::ptrdiff_t>(i));
            return x;
        }
    return json::Value{};
}

// Moves v[from] to v[to] within one object, when present.
void rename(json::Value& v, const std::string& from, const std::string& to)
{
    if (!child(v, from))
        return;
    put(v, to, take(v, from));
}

json::Value& sub(json::Value& v, const std::string& k)
{
    if (v.kind != json::Value::Object)
        v = obj();
    json::Value* c = child(v, k);
    if (!c)
    {
        v.obj.emplace_back(k, obj());
        c = &v.obj.back().second;
    }
    else if (c->kind != json::Value::Object)
        *c = obj();
    return *c;
}

// Version 4 keys are words separated by spaces; version 5 uses underscores (holo_file
// patch v4 -> v5). Applied to every key of a subtree.
void underscore_keys(json::Value& v)
{
    if (v.kind == json::Value::Array)
        for (auto& x : v.arr)
            underscore_keys(x);
    if (v.kind != json::Value::Object)
        return;
    for (auto& kv : v.obj)
    {
        for (char& c : kv.first)
            if (c == ' ')
                c = '_';
        underscore_keys(kv.second);
    }
}

const char* space_name(int i)
{
    static const char* n[] = {"NONE", "FRESNELTR", "ANGULARSP"};
    return i >= 0 && i <= 2 ? n[i] : "NONE";
}
const char* time_name(int i)
{
    static const char* n[] = {"NONE", "STFT", "PCA", "SSA_STFT"};
    return i >= 0 && i <= 3 ? n[i] : "NONE";
}

// The object at `path` under root, created (as empty objects) where missing. The returned
// reference is only valid until the next insertion into one of its ancestors: callers walk the
// path again for every access.
json::Value& path(json::Value& root, std::initializer_list<const char*> keys)
{
    json::Value* v = &root;
    for (const char* k : keys)
        v = &sub(*v, k);
    return *v;
}

// Versions 2 and 3: flat keys -> the version-4 nested layout (holo_file patch v3 -> v4 and its
// enum conversions: algorithm / time_filter were enum integers, mode was the computation + 1).
json::Value footer_v3_to_v4(json::Value& flat)
{
    json::Value out = obj();
    auto move_to = [&](const char* from, std::initializer_list<const char*> dst, const char* to) {
        json::Value x = take(flat, from);
        if (x.kind != json::Value::Null)
            put(path(out, dst), to, std::move(x));
    };
    move_to("#img", {"compute settings", "image rendering"}, "time transformation size");
    move_to("lambda", {"compute settings", "image rendering"}, "lambda");
    move_to("z", {"compute settings", "image rendering"}, "z distance");
    json::Value a = take(flat, "algorithm");
    if (a.kind == json::Value::Number)
        put(path(out, {"compute settings", "image rendering"}), "space transformation",
            str(space_name(static_cast<int>(a.num))));
    json::Value tf = take(flat, "time_filter");
    if (tf.kind == json::Value::Number)
        put(path(out, {"compute settings", "image rendering"}), "time transformation",
            str(time_name(static_cast<int>(tf.num))));
    json::Value mode = take(flat, "mode");
    if (mode.kind == json::Value::Number)
        put(path(out, {"compute settings", "image rendering"}), "image mode",
            str(static_cast<int>(mode.num) - 1 == 0 ? "RAW" : "HOLOGRAM"));
    move_to("fft_shift_enabled", {"compute settings", "view"}, "fft shift");
    move_to("renorm_enabled", {"compute settings", "view"}, "renorm");
    move_to("p", {"compute settings", "view", "p"}, "index");
    move_to("p_acc_level", {"compute settings", "view", "p"}, "accu level");
    move_to("contrast_max", {"compute settings", "view", "window", "xy", "contrast"}, "max");
    move_to("contrast_min", {"compute settings", "view", "window", "xy", "contrast"}, "min");
    move_to("img_acc_slice_xy_level", {"compute settings", "view", "window", "xy"}, "img accu level");
    move_to("log_scale", {"compute settings", "view", "window", "xy"}, "log enabled");
    put(path(out, {"info"}), "input fps", num(1));
    put(path(out, {"info"}), "contiguous", num(1));
    json::Value ps = take(flat, "pixel_size");
    if (ps.kind == json::Value::Number)
    {
        put(path(out, {"info", "pixel size"}), "x", ps);
        put(path(out, {"info", "pixel size"}), "y", ps);
    }
    return out;
}

// Version 4 -> 5 (holo_file patch v4 -> v5 and convert_v4_to_v5): underscored keys, the renamed
// view / window / info entries of this path, and two image-type spellings.
void footer_v4_to_v5(json::Value& f)
{
    if (child(f, "file info"))
    {
        rename(f, "file info", "info");
        put(path(f, {"info"}), "input fps", num(1));
        put(path(f, {"info"}), "contiguous", num(1));
    }
    rename(f, "compute settings", "compute_settings");
    underscore_keys(f);
    rename(path(f, {"compute_settings", "image_rendering"}), "z_distance", "propagation_distance");
    if (json::Value* f2 = child(path(f, {"compute_settings", "image_rendering"}), "filter2d"))
    {
        rename(*f2, "n1", "inner_radius");
        rename(*f2, "n2", "outer_radius");
    }
    rename(path(f, {"compute_settings", "view"}), "p", "z");
    rename(path(f, {"compute_settings", "view"}), "q", "z2");
    for (const char* k : {"z", "z2", "x", "y"})
        if (json::Value* a = child(path(f, {"compute_settings", "view"}), k))
        {
            rename(*a, "index", "start");
            rename(*a, "cuts", "start");
            rename(*a, "accu_level", "width");
        }
    rename(path(f, {"compute_settings", "view"}), "type", "image_type");
    if (json::Value* t = child(path(f, {"compute_settings", "view"}), "image_type"))
        if (t->kind == json::Value::String)
        {
            if (t->str == "PHASEINCREASE")
                t->str = "PHASE_INCREASE";
            else if (t->str == "SQUAREDMODULUS")
                t->str = "SQUARED_MODULUS";
        }
    if (json::Value* w = child(path(f, {"compute_settings", "view"}), "window"))
        for (const char* k : {"xy", "xz", "yz"})
            if (json::Value* a = child(*w, k))
            {
                rename(*a, "img_accu_level", "output_image_accumulation");
                rename(*a, "flip", "horizontal_flip");
                rename(*a, "rot", "rotation");
            }
    if (json::Value* c = child(path(f, {"compute_settings", "advanced"}), "contrast"))
        rename(*c, "cuts_p_offset", "frame_index_offset");
    rename(path(f, {"compute_settings"}), "composite", "color_composite_image");
    rename(path(f, {"info"}), "pixel_size", "pixel_pitch");
    if (child(path(f, {"info"}), "raw_bitshift"))
    {
        json::Value rb = take(path(f, {"info"}), "raw_bitshift");
        put(path(f, {"compute_settings", "advanced"}), "raw_bitshift", std::move(rb));
    }
}

}  // namespace

namespace hv {

// Converts a footer of `version` to the current layout in place; false when the version is newer
// than this build's (versions below 2 are read as 2, as the reference does).
bool holo_footer_convert(json::Value& footer, int version)
{
    if (version > kHoloVersion)
        return false;
    if (version < 2)
        version = 2;
    if (footer.kind != json::Value::Object)
        footer = obj();
    if (version <= 3)
        footer = footer_v3_to_v4(footer);
    if (version <= 4)
        footer_v4_to_v5(footer);
    // versions 5 and 6 share the current footer; the compute settings may still be version v0
    if (json::Value* cs = child(footer, "compute_settings"))
        if (!settings_convert_to_current(*cs))
            return false;
    return true;
}

}  // namespace hv

namespace {

hv_status copy_out(const std::string& s, char* buf, size_t cap, size_t* len)
{
    if (len)
        *len = s.size();
    if (!buf)
        return cap == 0 ? HV_OK : HV_INVALID_VALUE;
    if (cap < s.size() + 1)
    {
        set_last_error_msg("output buffer too small (see *len)");
        return HV_INVALID_VALUE;
    }
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return HV_OK;
}

}  // namespace

extern "C" {

hv_status hv_holo_open(const char* path, hv_holo_file** out)
{
    if (!path || !out)
        return HV_INVALID_VALUE;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f)
    {
        set_last_error_msg("cannot open the .holo file");
        return HV_FAILURE;
    }
    hv_holo_file* h = new (std::nothrow) hv_holo_file();
    if (!h)
    {
        std::fclose(f);
        return HV_FAILURE;
    }
    h->f = f;
    uint8_t raw[kHeaderBytes];
    if (std::fread(raw, 1, kHeaderBytes, f) != kHeaderBytes || std::memcmp(raw, "HOLO", 4) != 0)
    {
        set_last_error_msg("invalid .holo file: bad header");
        hv_holo_close(h);
        return HV_FAILURE;
    }
    decode_header(raw, h->hdr);
    if (h->hdr.bits_per_pixel == 0 || h->hdr.bits_per_pixel % 8 != 0 || h->hdr.width == 0 || h->hdr.height == 0)
    {
        set_last_error_msg("invalid .holo file: bad frame description");
        hv_holo_close(h);
        return HV_FAILURE;
    }
    h->frame_bytes = static_cast<uint64_t>(h->hdr.width) * h->hdr.height * (h->hdr.bits_per_pixel / 8);
    if (h->hdr.total_data_size != h->frame_bytes * h->hdr.img_nb)
    {
        set_last_error_msg("invalid .holo file: invalid total data size");
        hv_holo_close(h);
        return HV_FAILURE;
    }
    if (fseeko(f, 0, SEEK_END) != 0)
    {
        hv_holo_close(h);
        return HV_FAILURE;
    }
    const uint64_t size = static_cast<uint64_t>(ftello(f));
    const uint64_t footer_at = kHeaderBytes + h->hdr.total_data_size;
    if (size < footer_at)
    {
        set_last_error_msg("invalid .holo file: truncated frame data");
        hv_holo_close(h);
        return HV_FAILURE;
    }
    h->footer = obj();
    if (size > footer_at)
    {
        std::string text(static_cast<size_t>(size - footer_at), '\0');
        json::Value doc;
        std::string err;
        // like the reference, an unreadable footer is skipped (the settings are not essential)
        if (seek(f, footer_at) && std::fread(&text[0], 1, text.size(), f) == text.size() &&
            json::parse(text.c_str(), doc, err) && doc.kind == json::Value::Object)
        {
            if (!holo_footer_convert(doc, h->hdr.version))
            {
                set_last_error_msg("unsupported .holo version");
                hv_holo_close(h);
                return HV_ERR_UNSUPPORTED;
            }
            h->footer = std::move(doc);
            h->has_footer = true;
        }
    }
    *out = h;
    return HV_OK;
}

void hv_holo_close(hv_holo_file* h)
{
    if (!h)
        return;
    if (h->f)
        std::fclose(h->f);
    delete h;
}

hv_status hv_holo_get_header(const hv_holo_file* h, hv_holo_header* hdr, hv_frame_desc* fd)
{
    if (!h)
        return HV_INVALID_VALUE;
    if (hdr)
        *hdr = h->hdr;
    if (fd)
    {
        fd->width = h->hdr.width;
        fd->height = h->hdr.height;
        fd->depth = h->hdr.bits_per_pixel / 8;
        fd->byte_endian = h->hdr.endianness ? 1 : 0;
    }
    return HV_OK;
}

hv_status hv_holo_read_frames(hv_holo_file* h, uint64_t first, uint64_t n, void* dst)
{
    if (!h || (!dst && n))
        return HV_INVALID_VALUE;
    if (first > h->hdr.img_nb || n > h->hdr.img_nb - first)
    {
        set_last_error_msg("frame range past the end of the .holo file");
        return HV_INVALID_VALUE;
    }
    if (n == 0)
        return HV_OK;
    if (!seek(h->f, kHeaderBytes + first * h->frame_bytes) ||
        std::fread(dst, 1, static_cast<size_t>(n * h->frame_bytes), h->f) != n * h->frame_bytes)
    {
        set_last_error_msg("cannot read the .holo frames");
        return HV_FAILURE;
    }
    return HV_OK;
}

hv_status hv_holo_get_footer(const hv_holo_file* h, char* buf, size_t cap, size_t* len)
{
    if (!h)
        return HV_INVALID_VALUE;
    std::string s;
    json::dump(h->footer, s);
    return copy_out(s, buf, cap, len);
}

hv_status hv_holo_get_settings(const hv_holo_file* h, hv_settings* s)
{
    if (!h || !s)
        return HV_INVALID_VALUE;
    if (!h->has_footer)
        return HV_NO_IN_DATA;
    json::Value& footer = const_cast<json::Value&>(h->footer);
    if (json::Value* cs = child(footer, "compute_settings"))
    {
        hv_status r = settings_from_value(*cs, s, true);
        if (r != HV_OK)
            return r;
    }
    if (json::Value* info = child(footer, "info"))
    {
        if (json::Value* pp = child(*info, "pixel_pitch"))
            if (json::Value* x = child(*pp, "x"))
                if (x->kind == json::Value::Number)
                    s->pixel_size = static_cast<float>(x->num);  // pixels are square
        // camera_fps defaults to input_fps (InputHoloFile::import_info)
        json::Value* fps = child(*info, "camera_fps");
        if (!fps || fps->kind != json::Value::Number)
            fps = child(*info, "input_fps");
        if (fps && fps->kind == json::Value::Number)
            s->camera_fps = static_cast<int32_t>(fps->num);
    }
    return HV_OK;
}

hv_status hv_holo_create(const char* path, const hv_frame_desc* fd, int data_type, hv_holo_writer** out)
{
    if (!path || !fd || !out || fd->width == 0 || fd->height == 0 || fd->depth == 0)
        return HV_INVALID_VALUE;
    *out = nullptr;
    FILE* f = std::fopen(path, "wb");
    if (!f)
    {
        set_last_error_msg("cannot create the .holo file");
        return HV_FAILURE;
    }
    hv_holo_writer* w = new (std::nothrow) hv_holo_writer();
    if (!w)
    {
        std::fclose(f);
        return HV_FAILURE;
    }
    w->f = f;
    std::memcpy(w->hdr.magic, "HOLO", 4);
    w->hdr.version = kHoloVersion;
    w->hdr.bits_per_pixel = static_cast<uint16_t>(fd->depth * 8);
    w->hdr.width = fd->width;
    w->hdr.height = fd->height;
    w->hdr.img_nb = 0;
    w->hdr.total_data_size = 0;
    w->hdr.endianness = fd->byte_endian ? 1 : 0;
    w->hdr.data_type = static_cast<uint8_t>(data_type);
    w->frame_bytes = static_cast<uint64_t>(fd->width) * fd->height * fd->depth;
    uint8_t raw[kHeaderBytes];
    encode_header(w->hdr, raw);
    if (std::fwrite(raw, 1, kHeaderBytes, f) != kHeaderBytes)
    {
        std::fclose(f);
        delete w;
        set_last_error_msg("cannot write the .holo header");
        return HV_FAILURE;
    }
    *out = w;
    return HV_OK;
}

hv_status hv_holo_write_frames(hv_holo_writer* w, const void* frames, uint64_t n)
{
    if (!w || (!frames && n))
        return HV_INVALID_VALUE;
    if (n && std::fwrite(frames, 1, static_cast<size_t>(n * w->frame_bytes), w->f) != n * w->frame_bytes)
    {
        set_last_error_msg("cannot write the .holo frames");
        return HV_FAILURE;
    }
    w->frames += n;
    return HV_OK;
}

hv_status hv_holo_finish(hv_holo_writer* w, const char* footer_json)
{
    if (!w)
        return HV_INVALID_VALUE;
    hv_status r = HV_OK;
    if (footer_json && *footer_json)
    {
        json::Value doc;
        std::string err, text;
        if (!json::parse(footer_json, doc, err))
        {
            set_last_error_msg(("invalid footer json: " + err).c_str());
            r = HV_INVALID_VALUE;
        }
        else
        {
            json::dump(doc, text);
            if (std::fwrite(text.data(), 1, text.size(), w->f) != text.size())
                r = HV_FAILURE;
        }
    }
    // the image count and data size of the header are the frames actually written
    w->hdr.img_nb = static_cast<uint32_t>(w->frames);
    w->hdr.total_data_size = w->frames * w->frame_bytes;
    uint8_t raw[kHeaderBytes];
    encode_header(w->hdr, raw);
    if (!seek(w->f, 0) || std::fwrite(raw, 1, kHeaderBytes, w->f) != kHeaderBytes)
        r = HV_FAILURE;
    if (std::fclose(w->f) != 0 && r == HV_OK)
        r = HV_FAILURE;
    delete w;
    if (r == HV_FAILURE)
        set_last_error_msg("cannot finish the .holo file");
    return r;
}

hv_status hv_holo_make_footer(const hv_settings* s, int input_fps, int camera_fps, char* buf, size_t cap, size_t* len)
{
    if (!s)
        return HV_INVALID_VALUE;
    json::Value footer = obj();
    json::Value cs;
    settings_to_value(s, cs);
    put(footer, "compute_settings", std::move(cs));
    json::Value info = obj();
    json::Value pp = obj();
    put(pp, "x", num(s->pixel_size));
    put(pp, "y", num(s->pixel_size));
    put(info, "pixel_pitch", std::move(pp));
    put(info, "input_fps", num(input_fps));
    put(info, "camera_fps", num(camera_fps ? camera_fps : input_fps));
    put(info, "contiguous", num(1));
    put(info, "holovibes_version", str(hv_version()));
    put(footer, "info", std::move(info));
    std::string text;
    json::dump(footer, text);
    return copy_out(text, buf, cap, len);
}

hv_status hv_settings_to_json(const hv_settings* s, char* buf, size_t cap, size_t* len)
{
    if (!s)
        return HV_INVALID_VALUE;
    json::Value doc;
    settings_to_value(s, doc);
    std::string text;
    json::dump(doc, text);
    return copy_out(text, buf, cap, len);
}

hv_status hv_settings_convert_json(const char* in, char* buf, size_t cap, size_t* len)
{
    if (!in)
        return HV_INVALID_VALUE;
    json::Value doc;
    std::string err;
    if (!json::parse(in, doc, err))
    {
        set_last_error_msg(("invalid json: " + err).c_str());
        return HV_FAILURE;
    }
    if (!settings_convert_to_current(doc))
    {
        set_last_error_msg("unknown compute settings version");
        return HV_FAILURE;
    }
    std::string text;
    json::dump(doc, text);
    return copy_out(text, buf, cap, len);
}

hv_status hv_holo_convert_footer(const char* footer_json, int version, char* buf, size_t cap, size_t* len)
{
    if (!footer_json)
        return HV_INVALID_VALUE;
    json::Value doc;
    std::string err;
    if (!json::parse(footer_json, doc, err))
    {
        set_last_error_msg(("invalid json: " + err).c_str());
        return HV_FAILURE;
    }
    if (!holo_footer_convert(doc, version))
    {
        set_last_error_msg("unsupported .holo version");
        return HV_ERR_UNSUPPORTED;
    }
    std::string text;
    json::dump(doc, text);
    return copy_out(text, buf, cap, len);
}

}  // extern "C"
