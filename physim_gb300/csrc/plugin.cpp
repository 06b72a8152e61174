// plugin.cpp -- the physim transform-plugin front door: the symbols physim's
// loader binds for a C plugin (physim-core/src/plugin/discover.rs:327-373,
// physim-core/src/plugin/transform.rs:32-134), for the astro crate's gravity
// elements astro, astro2 and simple_astro (astro/src/transformers.rs).
//
// Each element's init parses the JSON property object the way the
// reference's generated init does (physim-attribute/src/lib.rs:60-85): text
// that is not a JSON object gives NULL; `theta` and `e` are read with
// as_f64, `e` is made absolute, and unknown keys are ignored.  The GPU is not
// touched until the first transform, because physim instantiates every
// element once with "{}" while scanning plugins (discover.rs:375-393).
#include <dlfcn.h>

#include <atomic>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "physim_gb300.h"
#include "plugin_state.h"

namespace pg {

// ------------------------------------------------------------------------
// Thread-local last error (physim_gpu_last_error)
// ------------------------------------------------------------------------
static thread_local char g_last_error[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
}

const char *last_error() { return g_last_error; }

// ------------------------------------------------------------------------
// Minimal strict JSON reader (RFC 8259), enough to validate the property
// object and pull out numbers and strings.
// ------------------------------------------------------------------------
namespace json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    double number = 0.0;
    bool boolean = false;
    std::string str;
};

struct Parser {
    const char *p, *end;
    int depth = 0;

    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool lit(const char *s)
    {
        size_t k = strlen(s);
        if ((size_t)(end - p) < k || memcmp(p, s, k) != 0) return false;
        p += k;
        return true;
    }
    static int hex(char c)
    {
        if (c >= '0' && c <= '9') return c - '0';
        if (c >= 'a' && c <= 'f') return c - 'a' + 10;
        if (c >= 'A' && c <= 'F') return c - 'A' + 10;
        return -1;
    }
    static void utf8(std::string &out, unsigned cp)
    {
        if (cp < 0x80) {
            out += (char)cp;
        } else if (cp < 0x800) {
            out += (char)(0xC0 | (cp >> 6));
            out += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += (char)(0xE0 | (cp >> 12));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        } else {
            out += (char)(0xF0 | (cp >> 18));
            out += (char)(0x80 | ((cp >> 12) & 0x3F));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        }
    }
    bool u4(unsigned &cp)
    {
        if (end - p < 4) return false;
        cp = 0;
        for (int k = 0; k < 4; ++k) {
            int h = hex(p[k]);
            if (h < 0) return false;
            cp = cp * 16 + (unsigned)h;
        }
        p += 4;
        return true;
    }
    bool string(std::string &out)
    {
        if (p >= end || *p != '"') return false;
        ++p;
        while (p < end) {
            unsigned char c = (unsigned char)*p++;
            if (c == '"') return true;
            if (c < 0x20) return false;
            if (c != '\\') {
                out += (char)c;
                continue;
            }
            if (p >= end) return false;
            char esc = *p++;
            switch (esc) {
            case '"': out += '"'; break;
            case '\\': out += '\\'; break;
            case '/': out += '/'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'n': out += '\n'; break;
            case 'r': out += '\r'; break;
            case 't': out += '\t'; break;
            case 'u': {
                unsigned cp;
                if (!u4(cp)) return false;
                if (cp >= 0xD800 && cp <= 0xDBFF) {
                    unsigned lo;
                    if (end - p < 6 || p[0] != '\\' || p[1] != 'u') return false;
                    p += 2;
                    if (!u4(lo) || lo < 0xDC00 || lo > 0xDFFF) return false;
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                } else if (cp >= 0xDC00 && cp <= 0xDFFF) {
                    return false;
                }
                utf8(out, cp);
                break;
            }
            default: return false;
            }
        }
        return false;
    }
    bool number(double &out)
    {
        const char *s = p;
        if (p < end && *p == '-') ++p;
        if (p >= end) return false;
        if (*p == '0') {
            ++p;
        } else if (*p >= '1' && *p <= '9') {
            while (p < end && *p >= '0' && *p <= '9') ++p;
        } else {
            return false;
        }
        if (p < end && *p == '.') {
            ++p;
            if (p >= end || *p < '0' || *p > '9') return false;
            while (p < end && *p >= '0' && *p <= '9') ++p;
        }
        if (p < end && (*p == 'e' || *p == 'E')) {
            ++p;
            if (p < end && (*p == '+' || *p == '-')) ++p;
            if (p >= end || *p < '0' || *p > '9') return false;
            while (p < end && *p >= '0' && *p <= '9') ++p;
        }
        std::string text(s, p);
        char *tail = nullptr;
        out = strtod(text.c_str(), &tail);
        // serde_json rejects numbers that overflow f64.
        return tail && *tail == '\0' && isfinite(out);
    }
    bool value(Value &v, std::map<std::string, Value> *obj_out = nullptr)
    {
        if (++depth > 128) return false;
        ws();
        if (p >= end) return false;
        bool ok = false;
        if (*p == '{') {
            ++p;
            v.kind = Value::Object;
            ws();
            if (p < end && *p == '}') {
                ++p;
                ok = true;
            } else {
                for (;;) {
                    ws();
                    std::string key;
                    if (!string(key)) break;
                    ws();
                    if (p >= end || *p != ':') break;
                    ++p;
                    Value child;
                    if (!value(child)) break;
                    if (obj_out) (*obj_out)[key] = child;  // last duplicate wins
                    ws();
                    if (p < end && *p == ',') {
                        ++p;
                        continue;
                    }
                    if (p < end && *p == '}') {
                        ++p;
                        ok = true;
                    }
                    break;
                }
            }
        } else if (*p == '[') {
            ++p;
            v.kind = Value::Array;
            ws();
            if (p < end && *p == ']') {
                ++p;
                ok = true;
            } else {
                for (;;) {
                    Value child;
                    if (!value(child)) break;
                    ws();
                    if (p < end && *p == ',') {
                        ++p;
                        continue;
                    }
                    if (p < end && *p == ']') {
                        ++p;
                        ok = true;
                    }
                    break;
                }
            }
        } else if (*p == '"') {
            v.kind = Value::String;
            ok = string(v.str);
        } else if (*p == 't') {
            v.kind = Value::Bool;
            v.boolean = true;
            ok = lit("true");
        } else if (*p == 'f') {
            v.kind = Value::Bool;
            ok = lit("false");
        } else if (*p == 'n') {
            v.kind = Value::Null;
            ok = lit("null");
        } else {
            v.kind = Value::Number;
            ok = number(v.number);
        }
        --depth;
        return ok;
    }
};

// Parses a JSON object into its top-level members.  False for anything else.
bool parse_object(const uint8_t *text, size_t len, std::map<std::string, Value> &out)
{
    Parser ps{(const char *)text, (const char *)text + len};
    ps.ws();
    if (ps.p >= ps.end || *ps.p != '{') return false;
    Value root;
    if (!ps.value(root, &out)) return false;
    ps.ws();
    return ps.p == ps.end;
}

}  // namespace json

// ------------------------------------------------------------------------
// Message bus (physim-core/src/messages.rs:201-226)
// ------------------------------------------------------------------------
static void *g_bus_target = nullptr;
typedef void (*PostBusFn)(void *, CMessage);
static std::atomic<PhysimBusFn> g_bus_override{nullptr};

static void post_configuration(const void *sender)
{
    // transformers.rs:107-111,198-203,266-270: (Low, "energysink", "gravity").
    if (!g_bus_target) return;
    CMessage msg;
    msg.priority = PHYSIM_PRIORITY_LOW;
    msg.topic = "energysink";
    msg.message = "gravity";
    msg.sender_id = (uintptr_t)sender;
    msg.origin = PHYSIM_ORIGIN_C;  // the host must not free these strings
    if (PhysimBusFn own = g_bus_override.load()) {
        own(g_bus_target, &msg);
        return;
    }
    PostBusFn post = (PostBusFn)dlsym(RTLD_DEFAULT, "post_bus_callback");
    if (!post) return;
    post(g_bus_target, msg);
}

extern "C" int physim_gpu_set_bus_callback(PhysimBusFn fn)
{
    g_bus_override.store(fn);
    return PHYSIM_OK;
}

// ------------------------------------------------------------------------
// Elements
// ------------------------------------------------------------------------
static const char *kElementNames[3] = {"simple_astro", "astro2", "astro"};

static const char *kBlurbs[3] = {
    "Compute exact gravitational accelerations (GB300 direct sum)",
    "Compute approximate gravitational accelerations with the Barnes-Hut algorithm (octree, "
    "GB300)",
    "Compute approximate gravitational accelerations with the Barnes-Hut algorithm (quadtree, "
    "GB300)"};

static ElementState *element_new(int kind, const uint8_t *config, uintptr_t len)
{
    if (config == nullptr) return nullptr;
    std::map<std::string, json::Value> props;
    if (!json::parse_object(config, len, props)) return nullptr;
    ElementState *el = new (std::nothrow) ElementState();
    if (!el) return nullptr;
    el->kind = kind;
    auto num = [&](const char *key, double dflt) {
        auto it = props.find(key);
        if (it != props.end() && it->second.kind == json::Value::Number) return it->second.number;
        return dflt;
    };
    el->theta = num("theta", 1.0);
    el->e = fabs(num("e", 1.0));
    double leaf = num("leaf_size", 1.0);
    el->leaf_size = (leaf >= 1.0 && leaf <= 64.0) ? (int)leaf : 1;
    double dev = num("device", 0.0);
    el->device = (dev >= 0.0 && dev < 64.0) ? (int)dev : 0;
    auto it = props.find("traversal");
    el->traversal = PHYSIM_TRAVERSAL_EXACT;
    if (it != props.end() && it->second.kind == json::Value::String && it->second.str == "warp")
        el->traversal = PHYSIM_TRAVERSAL_WARP;
    auto qd = props.find("quadrupole");
    el->multipole = (qd != props.end() && qd->second.kind == json::Value::Bool &&
                     qd->second.boolean)
                        ? kMultipoleQuadrupole
                        : kMultipoleMonopole;
    const double ct = num("com_theta", 0.0);
    el->com_theta = ct > 0.0 ? ct : 0.0;
    return el;
}

[[noreturn]] static void fatal(int kind, const char *what)
{
    fprintf(stderr, "Problem encountered in the %s element's transform method: %s. Aborting\n",
            kElementNames[kind], what);
    fflush(stderr);
    abort();
}

static void element_transform(int kind, const void *obj, const Entity *state, uintptr_t n,
                              Acceleration *acc, uintptr_t n_acc)
{
    if (obj == nullptr) return;
    ElementState *el = (ElementState *)obj;
    if (n_acc < n) {
        // transformers.rs indexes accelerations[i] for every i < state.len().
        if (getenv("PHYSIM_GB300_NO_ABORT")) {
            set_error("acceleration_len %zu < state_len %zu", (size_t)n_acc, (size_t)n);
            fprintf(stderr, "%s transform: %s\n", kElementNames[kind], last_error());
            return;
        }
        fatal(kind, "index out of bounds: acceleration_len < state_len");
    }
    int rc = element_accumulate(el, state, (size_t)n, acc);
    if (rc != PHYSIM_OK) {
        if (getenv("PHYSIM_GB300_NO_ABORT")) {
            fprintf(stderr, "%s transform: %s\n", kElementNames[kind], last_error());
            return;
        }
        fatal(kind, last_error());
    }
}

static char *element_descriptions(int kind, void *obj, RustStringAllocFn alloc)
{
    if (obj == nullptr || alloc == nullptr) return nullptr;
    std::string s = "{";
    if (kind != 0) {
        s += "\"theta\":\"Barnes-Hut parameter. Increase for speed, decrease for accuracy. "
             "Default=1.0\",";
        s += "\"leaf_size\":\"Bodies per tree leaf on the GPU (1..64). 1 reproduces the "
             "reference tree. Default=1\",";
        s += "\"traversal\":\"exact: every body uses its own interaction list; warp: a cell is "
             "accepted only when all 32 bodies of a warp accept it. Default=exact\",";
        s += "\"quadrupole\":\"true adds each accepted cell's quadrupole moment to its "
             "monopole. Default=false\",";
        s += "\"com_theta\":\"If > 0, a cell is also opened unless its bodies lie within "
             "com_theta times the distance to its centre of mass. Default=0 (off)\",";
    }
    s += "\"e\":\"Easing factor. Modify G*Ma*Mb*(r-e)^-2. Default=1.0\",";
    s += "\"device\":\"CUDA device ordinal. Default=0\"}";
    return alloc(s.c_str());
}

static ElementMetaFFI element_register(int kind, RustStringAllocFn alloc)
{
    ElementMetaFFI meta;
    meta.kind = PHYSIM_KIND_TRANSFORM;
    meta.name = alloc(kElementNames[kind]);
    meta.plugin = alloc("physim_gb300");
    meta.version = alloc("0.1.0");
    meta.license = alloc("MIT");
    meta.author = alloc("physim-gb300 contributors");
    meta.blurb = alloc(kBlurbs[kind]);
    meta.repo = alloc("");
    return meta;
}

}  // namespace pg

using namespace pg;

extern "C" {

const char *get_plugin_abi_info(void) { return "C"; }

const char *register_plugin(void) { return "astro,astro2,simple_astro"; }

void set_callback_target(void *target)
{
    if (target == nullptr) {
        fprintf(stderr, "Error: callback target is null\n");
        abort();
    }
    g_bus_target = target;
}

const char *physim_gpu_last_error(void) { return pg::last_error(); }

#define PG_ELEMENT_EXPORTS(NAME, KIND)                                                      \
    void *NAME##_init(const uint8_t *config, uintptr_t len)                                 \
    {                                                                                       \
        return (void *)element_new(KIND, config, len);                                      \
    }                                                                                       \
    void NAME##_transform(const void *obj, const Entity *state, uintptr_t state_len,        \
                          Acceleration *acc, uintptr_t acc_len)                             \
    {                                                                                       \
        element_transform(KIND, obj, state, state_len, acc, acc_len);                       \
    }                                                                                       \
    void NAME##_destroy(void *obj)                                                          \
    {                                                                                       \
        if (obj) element_destroy((ElementState *)obj);                                      \
    }                                                                                       \
    char *NAME##_get_property_descriptions(void *obj, RustStringAllocFn alloc)              \
    {                                                                                       \
        return element_descriptions(KIND, obj, alloc);                                      \
    }                                                                                       \
    void NAME##_recv_message(void *obj, const CMessage *msg)                                \
    {                                                                                       \
        (void)obj;                                                                          \
        (void)msg;                                                                          \
    }                                                                                       \
    void NAME##_post_configuration_messages(void *obj)                                      \
    {                                                                                       \
        if (obj) post_configuration(obj);                                                   \
    }                                                                                       \
    const TransformElementAPI *NAME##_get_api(void)                                         \
    {                                                                                       \
        static const TransformElementAPI api = {                                            \
            NAME##_init,         NAME##_transform,    NAME##_destroy,                       \
            NAME##_get_property_descriptions, NAME##_recv_message,                          \
            NAME##_post_configuration_messages};                                            \
        return &api;                                                                        \
    }                                                                                       \
    ElementMetaFFI NAME##_register(RustStringAllocFn alloc)                                 \
    {                                                                                       \
        return element_register(KIND, alloc);                                               \
    }

PG_ELEMENT_EXPORTS(simple_astro, 0)
PG_ELEMENT_EXPORTS(astro2, 1)
PG_ELEMENT_EXPORTS(astro, 2)

}  // extern "C"
