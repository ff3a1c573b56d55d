// preset.cpp - the reference's preset files: parse, apply to a world, write.
//
// Format and semantics of CellFlowWidget::loadPreset / savePreset
// (cuda-native/src/CellFlowWidget.cpp:1070-1180 and :1182-1259): one JSON
// object with the reference's keys.  Loading sets the particle count and the
// type count (each respawns, :1079-1084), the parameters present, the
// per-type radius values (:1155-1166), the raw force table (:1168-1175) and
// then transforms the table with forceRange / forceBias / forceOffset
// (:1178).  Rendering keys (point size, depth fade, DOF, camera, effect) are
// kept as text so a preset written back keeps them.
//
// The JSON reader is this library's own: objects, arrays, strings (with the
// escapes of RFC 8259), numbers, true / false / null; numbers are read with
// std::from_chars, independent of the C locale.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cf_internal.hpp"

namespace cf {
int fail(int code, const std::string& msg);
}

namespace {

struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JValue> items;                           // Array
    std::vector<std::pair<std::string, JValue>> fields;  // Object, in file order
    std::string raw;                                     // the value's text (for keys kept as text)
};

class Reader {
public:
    Reader(const char* s, size_t n) : p_(s), begin_(s), end_(s + n) {}

    bool parse(JValue& out, std::string& err)
    {
        skip();
        if (!value(out, 0)) {
            err = err_ + " at offset " + std::to_string(p_ - begin_);
            return false;
        }
        skip();
        if (p_ != end_) {
            err = "trailing characters at offset " + std::to_string(p_ - begin_);
            return false;
        }
        return true;
    }

private:
    const char* p_;
    const char* begin_;
    const char* end_;
    std::string err_;

    bool bad(const char* what)
    {
        err_ = what;
        return false;
    }
    void skip()
    {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) p_++;
    }
    bool lit(const char* w)
    {
        const size_t n = std::strlen(w);
        if ((size_t)(end_ - p_) < n || std::memcmp(p_, w, n) != 0) return false;
        p_ += n;
        return true;
    }
    static void utf8(std::string& s, unsigned cp)
    {
        if (cp < 0x80) {
            s += (char)cp;
        } else if (cp < 0x800) {
            s += (char)(0xC0 | (cp >> 6));
            s += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            s += (char)(0xE0 | (cp >> 12));
            s += (char)(0x80 | ((cp >> 6) & 0x3F));
            s += (char)(0x80 | (cp & 0x3F));
        } else {
            s += (char)(0xF0 | (cp >> 18));
            s += (char)(0x80 | ((cp >> 12) & 0x3F));
            s += (char)(0x80 | ((cp >> 6) & 0x3F));
            s += (char)(0x80 | (cp & 0x3F));
        }
    }
    bool hex4(unsigned& v)
    {
        if (end_ - p_ < 4) return bad("truncated \\u escape");
        v = 0;
        for (int k = 0; k < 4; k++) {
            const char c = *p_++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
            else return bad("bad \\u escape");
        }
        return true;
    }
    bool string(std::string& s)
    {
        if (p_ >= end_ || *p_ != '"') return bad("expected a string");
        p_++;
        while (true) {
            if (p_ >= end_) return bad("unterminated string");
            const char c = *p_++;
            if (c == '"') return true;
            if ((unsigned char)c < 0x20) return bad("control character in a string");
            if (c != '\\') {
                s += c;
                continue;
            }
            if (p_ >= end_) return bad("unterminated escape");
            const char e = *p_++;
            switch (e) {
            case '"': s += '"'; break;
            case '\\': s += '\\'; break;
            case '/': s += '/'; break;
            case 'b': s += '\b'; break;
            case 'f': s += '\f'; break;
            case 'n': s += '\n'; break;
            case 'r': s += '\r'; break;
            case 't': s += '\t'; break;
            case 'u': {
                unsigned cp;
                if (!hex4(cp)) return false;
                if (cp >= 0xD800 && cp < 0xDC00) {  // surrogate pair
                    unsigned lo;
                    if (!lit("\\u") || !hex4(lo) || lo < 0xDC00 || lo >= 0xE000) return bad("bad surrogate pair");
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                }
                utf8(s, cp);
                break;
            }
            default: return bad("bad escape");
            }
        }
    }
    bool number(double& v)
    {
        const char* s = p_;
        if (p_ < end_ && *p_ == '-') p_++;
        if (p_ >= end_ || !(*p_ >= '0' && *p_ <= '9')) return bad("bad number");
        if (*p_ == '0') p_++;
        else
            while (p_ < end_ && *p_ >= '0' && *p_ <= '9') p_++;
        if (p_ < end_ && *p_ == '.') {
            p_++;
            if (p_ >= end_ || !(*p_ >= '0' && *p_ <= '9')) return bad("bad fraction");
            while (p_ < end_ && *p_ >= '0' && *p_ <= '9') p_++;
        }
        if (p_ < end_ && (*p_ == 'e' || *p_ == 'E')) {
            p_++;
            if (p_ < end_ && (*p_ == '+' || *p_ == '-')) p_++;
            if (p_ >= end_ || !(*p_ >= '0' && *p_ <= '9')) return bad("bad exponent");
            while (p_ < end_ && *p_ >= '0' && *p_ <= '9') p_++;
        }
        const auto r = std::from_chars(s, p_, v);
        if (r.ec != std::errc() || r.ptr != p_) return bad("number out of range");
        return true;
    }
    bool value(JValue& v, int depth)
    {
        if (depth > 64) return bad("nesting too deep");
        skip();
        const char* start = p_;
        if (p_ >= end_) return bad("unexpected end");
        bool ok = true;
        switch (*p_) {
        case '{': {
            v.kind = JValue::Object;
            p_++;
            skip();
            if (p_ < end_ && *p_ == '}') {
                p_++;
                break;
            }
            while (true) {
                skip();
                std::string key;
                if (!string(key)) return false;
                skip();
                if (p_ >= end_ || *p_ != ':') return bad("expected ':'");
                p_++;
                JValue child;
                if (!value(child, depth + 1)) return false;
                v.fields.emplace_back(std::move(key), std::move(child));
                skip();
                if (p_ < end_ && *p_ == ',') {
                    p_++;
                    continue;
                }
                if (p_ < end_ && *p_ == '}') {
                    p_++;
                    break;
                }
                return bad("expected ',' or '}'");
            }
            break;
        }
        case '[': {
            v.kind = JValue::Array;
            p_++;
            skip();
            if (p_ < end_ && *p_ == ']') {
                p_++;
                break;
            }
            while (true) {
                JValue child;
                if (!value(child, depth + 1)) return false;
                v.items.push_back(std::move(child));
                skip();
                if (p_ < end_ && *p_ == ',') {
                    p_++;
                    continue;
                }
                if (p_ < end_ && *p_ == ']') {
                    p_++;
                    break;
                }
                return bad("expected ',' or ']'");
            }
            break;
        }
        case '"':
            v.kind = JValue::String;
            ok = string(v.str);
            break;
        case 't':
            v.kind = JValue::Bool;
            v.b = true;
            ok = lit("true") || bad("bad literal");
            break;
        case 'f':
            v.kind = JValue::Bool;
            ok = lit("false") || bad("bad literal");
            break;
        case 'n':
            v.kind = JValue::Null;
            ok = lit("null") || bad("bad literal");
            break;
        default:
            v.kind = JValue::Number;
            ok = number(v.num);
        }
        if (ok) v.raw.assign(start, p_);
        return ok;
    }
};

// QJsonValue::toDouble / toInt of the reference: numbers convert, anything
// else gives 0 (toInt also gives 0 for a non-integral number).
double to_double(const JValue& v) { return v.kind == JValue::Number ? v.num : 0.0; }
int to_int(const JValue& v)
{
    if (v.kind != JValue::Number || v.num != std::floor(v.num) || std::fabs(v.num) > 2147483647.0) return 0;
    return (int)v.num;
}

struct FloatKey {
    const char* key;
    int bit;
};

// Shortest text that reads back as the same double (Qt writes doubles so).
std::string num_text(double v)
{
    if (!std::isfinite(v)) return "null";  // JSON has no inf / nan
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof(buf), v);
    return std::string(buf, r.ptr);
}

void append_json_string(std::string& out, const std::string& s)
{
    out += '"';
    for (unsigned char c : s) {
        switch (c) {
        case '"': out += "\\\""; break;
        case '\\': out += "\\\\"; break;
        case '\n': out += "\\n"; break;
        case '\r': out += "\\r"; break;
        case '\t': out += "\\t"; break;
        case '\b': out += "\\b"; break;
        case '\f': out += "\\f"; break;
        default:
            if (c < 0x20) {
                char b[8];
                std::snprintf(b, sizeof(b), "\\u%04x", c);
                out += b;
            } else {
                out += (char)c;
            }
        }
    }
    out += '"';
}

}  // namespace

extern "C" {

int cf_preset_parse(const char* json, size_t len, cf_preset* out)
{
    using cf::fail;
    if (!json || !out) return fail(CF_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof(*out));
    Reader rd(json, len);
    JValue root;
    std::string err;
    if (!rd.parse(root, err)) return fail(CF_ERR_INVALID, "preset JSON: " + err);
    if (root.kind != JValue::Object) return fail(CF_ERR_INVALID, "preset JSON: the top level is not an object");
    cf_default_params(&out->params);
    out->force_range = 0.28f;  // SimulationParams defaults (SimulationParams.h:32-37)
    out->force_bias = -0.20f;
    out->force_offset = 1.0f;
    out->lfo_s = 0.1f;
    std::string extra;  // keys this library does not interpret, kept as text
    for (const auto& kv : root.fields) {
        const std::string& k = kv.first;
        const JValue& v = kv.second;
        auto setf = [&](float* dst, unsigned bit) {
            *dst = (float)to_double(v);
            out->present |= bit;
        };
        if (k == "PARTICLE_COUNT") {
            out->particle_count = to_int(v);
            out->present |= CF_PRESET_PARTICLE_COUNT;
        } else if (k == "numParticleTypes") {
            out->params.num_particle_types = to_int(v);
            out->present |= CF_PRESET_NUM_TYPES;
        } else if (k == "radius") setf(&out->params.radius, CF_PRESET_RADIUS);
        else if (k == "delta_t") setf(&out->params.delta_t, CF_PRESET_DELTA_T);
        else if (k == "friction") setf(&out->params.friction, CF_PRESET_FRICTION);
        else if (k == "repulsion") setf(&out->params.repulsion, CF_PRESET_REPULSION);
        else if (k == "attraction") setf(&out->params.attraction, CF_PRESET_ATTRACTION);
        else if (k == "k") setf(&out->params.k, CF_PRESET_K);
        else if (k == "balance") setf(&out->params.balance, CF_PRESET_BALANCE);
        else if (k == "forceMultiplier") setf(&out->params.force_multiplier, CF_PRESET_FORCE_MULTIPLIER);
        else if (k == "canvasWidth") setf(&out->params.canvas_width, CF_PRESET_CANVAS);
        else if (k == "canvasHeight") setf(&out->params.canvas_height, CF_PRESET_CANVAS);
        else if (k == "canvasDepth") setf(&out->params.canvas_depth, CF_PRESET_CANVAS);
        else if (k == "forceRange") setf(&out->force_range, CF_PRESET_FORCE_TRANSFORM);
        else if (k == "forceBias") setf(&out->force_bias, CF_PRESET_FORCE_TRANSFORM);
        else if (k == "forceOffset") setf(&out->force_offset, CF_PRESET_FORCE_TRANSFORM);
        else if (k == "ratio") setf(&out->ratio, CF_PRESET_LFO);
        else if (k == "lfoA") setf(&out->lfo_a, CF_PRESET_LFO);
        else if (k == "lfoS") setf(&out->lfo_s, CF_PRESET_LFO);
        else if (k == "spawnRegionSize") setf(&out->spawn_region, CF_PRESET_SPAWN_REGION);
        else if (k == "radioByType") {
            out->present |= CF_PRESET_RADIO;
            for (const auto& x : v.items)
                if (out->n_radio < CF_MAX_TYPES) out->radio[out->n_radio++] = (float)to_double(x);
        } else if (k == "rawForceTable") {
            out->present |= CF_PRESET_RAW_TABLE;
            for (const auto& x : v.items)
                if (out->n_raw < CF_MAX_TYPES * CF_MAX_TYPES) out->raw[out->n_raw++] = (float)to_double(x);
        } else if (k == "particleColors") {
            out->present |= CF_PRESET_COLORS;
            for (const auto& x : v.items) {
                if (out->n_colors >= CF_MAX_TYPES) break;
                cf_color c{0.0f, 0.0f, 0.0f};
                for (const auto& f : x.fields) {
                    if (f.first == "r") c.r = (float)to_double(f.second);
                    if (f.first == "g") c.g = (float)to_double(f.second);
                    if (f.first == "b") c.b = (float)to_double(f.second);
                }
                out->colors[out->n_colors++] = c;
            }
        } else {
            if (!extra.empty()) extra += ",\n";
            extra += "    ";
            append_json_string(extra, k);
            extra += ": ";
            extra += v.raw;
        }
    }
    if (extra.size() >= sizeof(out->extra)) return fail(CF_ERR_CAPACITY, "preset JSON: too many uninterpreted keys");
    std::memcpy(out->extra, extra.c_str(), extra.size() + 1);
    return CF_OK;
}

int cf_preset_apply(cf_world* w, const cf_preset* p, uint64_t seed, cf_step_params* params)
{
    using cf::fail;
    if (!w || !p) return fail(CF_ERR_INVALID, "null argument");
    int rc = CF_OK;
    // CellFlowWidget.cpp:1079-1084: particle count, then type count (each respawns)
    if (p->present & CF_PRESET_PARTICLE_COUNT) {
        if (p->particle_count < 0) return fail(CF_ERR_INVALID, "PARTICLE_COUNT must be >= 0");
        if ((rc = cf_set_particle_count(w, p->particle_count, seed))) return rc;
    }
    if (p->present & CF_PRESET_NUM_TYPES) {
        if ((rc = cf_set_num_particle_types(w, p->params.num_particle_types, seed))) return rc;
    }
    int T = 0;
    if ((rc = cf_num_particle_types(w, &T))) return rc;
    // :1155-1166: radioByType values for i < min(len, T)
    if (p->present & CF_PRESET_RADIO)
        for (int i = 0; i < p->n_radio && i < T; i++)
            if ((rc = cf_set_radio_by_type_value(w, i, p->radio[i]))) return rc;
    // :1168-1175: raw force table for i < min(len, T*T), the rest kept
    if (p->present & CF_PRESET_RAW_TABLE) {
        std::vector<float> raw((size_t)T * T);
        if ((rc = cf_get_raw_force_table(w, raw.data(), T * T))) return rc;
        for (int i = 0; i < p->n_raw && i < T * T; i++) raw[i] = p->raw[i];
        if ((rc = cf_set_raw_force_table(w, raw.data(), T * T))) return rc;
    }
    // :1178: the table transform with the preset's (or default) range, bias, offset
    if ((rc = cf_update_force_table(w, p->force_range, p->force_bias, p->force_offset))) return rc;
    if (params) {
        const cf_step_params& q = p->params;
        const unsigned m = p->present;
        if (m & CF_PRESET_RADIUS) params->radius = q.radius;
        if (m & CF_PRESET_DELTA_T) params->delta_t = q.delta_t;
        if (m & CF_PRESET_FRICTION) params->friction = q.friction;
        if (m & CF_PRESET_REPULSION) params->repulsion = q.repulsion;
        if (m & CF_PRESET_ATTRACTION) params->attraction = q.attraction;
        if (m & CF_PRESET_K) params->k = q.k;
        if (m & CF_PRESET_BALANCE) params->balance = q.balance;
        if (m & CF_PRESET_FORCE_MULTIPLIER) params->force_multiplier = q.force_multiplier;
        if (m & CF_PRESET_CANVAS) {
            params->canvas_width = q.canvas_width;
            params->canvas_height = q.canvas_height;
            params->canvas_depth = q.canvas_depth;
        }
        params->num_particle_types = T;
    }
    return CF_OK;
}

int cf_preset_write(cf_world* w, const cf_preset* p, char* buf, size_t cap, size_t* len)
{
    using cf::fail;
    if (!w || !p || !len) return fail(CF_ERR_INVALID, "null argument");
    int rc = CF_OK, n = 0, T = 0;
    if ((rc = cf_particle_count(w, &n)) || (rc = cf_num_particle_types(w, &T))) return rc;
    std::vector<float> radio(T), raw((size_t)T * T);
    if ((rc = cf_get_radio_by_type(w, radio.data(), T))) return rc;
    if ((rc = cf_get_raw_force_table(w, raw.data(), T * T))) return rc;
    const cf_step_params& q = p->params;
    // key order and set of CellFlowWidget::savePreset (:1182-1259); the world
    // supplies the count, the types, the radius values and the raw table
    std::string s = "{\n";
    auto kv = [&](const char* k, const std::string& v) {
        s += "    \"";
        s += k;
        s += "\": ";
        s += v;
        s += ",\n";
    };
    kv("PARTICLE_COUNT", std::to_string(n));
    kv("numParticleTypes", std::to_string(T));
    kv("radius", num_text(q.radius));
    kv("delta_t", num_text(q.delta_t));
    kv("friction", num_text(q.friction));
    kv("repulsion", num_text(q.repulsion));
    kv("attraction", num_text(q.attraction));
    kv("k", num_text(q.k));
    kv("balance", num_text(q.balance));
    kv("forceMultiplier", num_text(q.force_multiplier));
    kv("forceRange", num_text(p->force_range));
    kv("forceBias", num_text(p->force_bias));
    kv("ratio", num_text(p->ratio));
    kv("lfoA", num_text(p->lfo_a));
    kv("lfoS", num_text(p->lfo_s));
    kv("forceOffset", num_text(p->force_offset));
    kv("canvasWidth", num_text(q.canvas_width));
    kv("canvasHeight", num_text(q.canvas_height));
    kv("canvasDepth", num_text(q.canvas_depth));
    if (p->present & CF_PRESET_SPAWN_REGION) kv("spawnRegionSize", num_text(p->spawn_region));
    if (p->extra[0]) {
        s += p->extra;
        s += ",\n";
    }
    std::string colors = "[";
    for (int i = 0; i < p->n_colors && i < T; i++) {
        if (i) colors += ", ";
        colors += "{\"b\": " + num_text(p->colors[i].b) + ", \"g\": " + num_text(p->colors[i].g) +
                  ", \"r\": " + num_text(p->colors[i].r) + "}";
    }
    kv("particleColors", colors + "]");
    std::string rb = "[";
    for (int i = 0; i < T; i++) rb += (i ? ", " : "") + num_text(radio[i]);
    kv("radioByType", rb + "]");
    std::string rt = "[";
    for (int i = 0; i < T * T; i++) rt += (i ? ", " : "") + num_text(raw[i]);
    s += "    \"rawForceTable\": " + rt + "]\n}\n";
    *len = s.size();
    if (!buf) return CF_OK;  // size query
    if (cap < s.size() + 1) return fail(CF_ERR_CAPACITY, "buffer smaller than the preset text");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return CF_OK;
}

}  // extern "C"
