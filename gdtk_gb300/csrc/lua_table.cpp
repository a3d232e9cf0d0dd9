// lua_table.cpp -- see lua_table.h.
#include "lua_table.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace gdtk {

namespace {

const LuaValue kNil;

std::string num_key(double v) {
    if (v != std::floor(v)) throw std::runtime_error("non-integer number used as a table key");
    return "#" + std::to_string((long)v);
}

struct Tok {
    enum T { END, NUM, STR, NAME, OP } t;
    std::string s;
    double v = 0;
};

class Lexer {
public:
    explicit Lexer(const std::string& src) : s_(src) {}
    std::vector<Tok> run() {
        std::vector<Tok> out;
        while (true) {
            skip();
            if (i_ >= s_.size()) { out.push_back({Tok::END, "", 0}); return out; }
            char c = s_[i_];
            if (std::isdigit((unsigned char)c) || (c == '.' && i_ + 1 < s_.size() && std::isdigit((unsigned char)s_[i_ + 1]))) {
                const char* b = s_.c_str() + i_;
                char* e = nullptr;
                double v = std::strtod(b, &e);
                if (e == b) throw std::runtime_error("bad number in Lua input");
                out.push_back({Tok::NUM, std::string(b, e - b), v});
                i_ += (size_t)(e - b);
            } else if (c == '\'' || c == '"') {
                char q = c; ++i_;
                std::string v;
                while (i_ < s_.size() && s_[i_] != q) {
                    if (s_[i_] == '\\' && i_ + 1 < s_.size()) {
                        char n = s_[i_ + 1];
                        v.push_back(n == 'n' ? '\n' : n == 't' ? '\t' : n);
                        i_ += 2;
                    } else {
                        v.push_back(s_[i_++]);
                    }
                }
                if (i_ >= s_.size()) throw std::runtime_error("unterminated string in Lua input");
                ++i_;
                out.push_back({Tok::STR, v, 0});
            } else if (std::isalpha((unsigned char)c) || c == '_') {
                size_t b = i_;
                while (i_ < s_.size() && (std::isalnum((unsigned char)s_[i_]) || s_[i_] == '_')) ++i_;
                out.push_back({Tok::NAME, s_.substr(b, i_ - b), 0});
            } else if (std::string("=,;{}[]().-+*/").find(c) != std::string::npos) {
                out.push_back({Tok::OP, std::string(1, c), 0});
                ++i_;
            } else {
                throw std::runtime_error(std::string("unexpected character in Lua input: ") + c);
            }
        }
    }

private:
    void skip() {
        while (i_ < s_.size()) {
            if (std::isspace((unsigned char)s_[i_])) { ++i_; continue; }
            if (s_.compare(i_, 2, "--") == 0) {
                size_t j = i_ + 2;
                if (j < s_.size() && s_[j] == '[') {   // long comment --[==[ ... ]==]
                    size_t k = j + 1; int eq = 0;
                    while (k < s_.size() && s_[k] == '=') { ++eq; ++k; }
                    if (k < s_.size() && s_[k] == '[') {
                        std::string close = "]" + std::string(eq, '=') + "]";
                        size_t e = s_.find(close, k + 1);
                        if (e == std::string::npos) throw std::runtime_error("unterminated long comment");
                        i_ = e + close.size();
                        continue;
                    }
                }
                while (i_ < s_.size() && s_[i_] != '\n') ++i_;
                continue;
            }
            break;
        }
    }
    const std::string& s_;
    size_t i_ = 0;
};

class Parser {
public:
    explicit Parser(std::vector<Tok> t) : t_(std::move(t)) {
        env_.kind = LuaValue::TABLE;
        env_.tab = std::make_shared<std::map<std::string, LuaValue>>();
    }
    LuaValue chunk() {
        while (peek().t != Tok::END) {
            if (peek().t == Tok::OP && peek().s == ";") { ++i_; continue; }
            statement();
        }
        return env_;
    }

private:
    const Tok& peek(size_t o = 0) const { return t_[std::min(i_ + o, t_.size() - 1)]; }
    Tok take() { return t_[i_++]; }
    void expect(const std::string& op) {
        if (peek().t != Tok::OP || peek().s != op) throw std::runtime_error("expected '" + op + "' in Lua input");
        ++i_;
    }
    static std::string key_of(const LuaValue& k) {
        if (k.kind == LuaValue::NUMBER) return num_key(k.num);
        if (k.kind == LuaValue::STRING) return k.str;
        throw std::runtime_error("unsupported table key type");
    }
    void statement() {
        Tok name = take();
        if (name.t != Tok::NAME) throw std::runtime_error("statement must begin with a name");
        std::vector<std::string> keys;
        while (peek().t == Tok::OP && (peek().s == "." || peek().s == "[")) {
            if (take().s == ".") {
                Tok f = take();
                if (f.t != Tok::NAME) throw std::runtime_error("expected field name");
                keys.push_back(f.s);
            } else {
                keys.push_back(key_of(expr()));
                expect("]");
            }
        }
        expect("=");
        LuaValue v = expr();
        if (keys.empty()) { (*env_.tab)[name.s] = v; return; }
        auto it = env_.tab->find(name.s);
        if (it == env_.tab->end() || it->second.kind != LuaValue::TABLE)
            throw std::runtime_error("assignment into undefined table " + name.s);
        LuaValue* target = &it->second;
        for (size_t k = 0; k + 1 < keys.size(); ++k) {
            auto jt = target->tab->find(keys[k]);
            if (jt == target->tab->end() || jt->second.kind != LuaValue::TABLE)
                throw std::runtime_error("assignment into undefined table field " + keys[k]);
            target = &jt->second;
        }
        (*target->tab)[keys.back()] = v;
    }
    LuaValue expr() {
        const Tok& tk = peek();
        LuaValue v;
        if (tk.t == Tok::OP && tk.s == "-") {
            ++i_;
            v = expr();
            if (v.kind != LuaValue::NUMBER) throw std::runtime_error("unary minus on a non-number");
            v.num = -v.num;
            return v;
        }
        if (tk.t == Tok::OP && tk.s == "{") return table();
        Tok t = take();
        switch (t.t) {
        case Tok::NUM: v.kind = LuaValue::NUMBER; v.num = t.v; return v;
        case Tok::STR: v.kind = LuaValue::STRING; v.str = t.s; return v;
        case Tok::NAME:
            if (t.s == "true") { v.kind = LuaValue::BOOL; v.b = true; return v; }
            if (t.s == "false") { v.kind = LuaValue::BOOL; v.b = false; return v; }
            if (t.s == "nil") return v;
            {
                auto it = env_.tab->find(t.s);
                if (it == env_.tab->end()) throw std::runtime_error("undefined name " + t.s);
                return it->second;
            }
        default: break;
        }
        throw std::runtime_error("unexpected token '" + t.s + "' in Lua input");
    }
    LuaValue table() {
        expect("{");
        LuaValue out;
        out.kind = LuaValue::TABLE;
        out.tab = std::make_shared<std::map<std::string, LuaValue>>();
        long n = 1;
        while (!(peek().t == Tok::OP && peek().s == "}")) {
            if (peek().t == Tok::OP && peek().s == "[") {
                ++i_;
                std::string k = key_of(expr());
                expect("]");
                expect("=");
                (*out.tab)[k] = expr();
            } else if (peek().t == Tok::NAME && peek(1).t == Tok::OP && peek(1).s == "=") {
                std::string k = take().s;
                ++i_;
                (*out.tab)[k] = expr();
            } else {
                (*out.tab)["#" + std::to_string(n++)] = expr();
            }
            if (peek().t == Tok::OP && (peek().s == "," || peek().s == ";")) ++i_;
            else if (!(peek().t == Tok::OP && peek().s == "}")) throw std::runtime_error("expected ',' or '}' in table");
        }
        expect("}");
        return out;
    }
    std::vector<Tok> t_;
    size_t i_ = 0;
    LuaValue env_;
};

}  // namespace

const LuaValue& LuaValue::get(const std::string& key) const {
    if (kind != TABLE) return kNil;
    auto it = tab->find(key);
    return it == tab->end() ? kNil : it->second;
}

const LuaValue& LuaValue::at(long index) const { return get("#" + std::to_string(index)); }

std::vector<long> LuaValue::int_keys() const {
    std::vector<long> keys;
    if (kind != TABLE) return keys;
    for (auto& kv : *tab)
        if (!kv.first.empty() && kv.first[0] == '#') keys.push_back(std::strtol(kv.first.c_str() + 1, nullptr, 10));
    std::sort(keys.begin(), keys.end());
    return keys;
}

std::vector<LuaValue> LuaValue::sequence() const {
    std::vector<LuaValue> out;
    for (long k : int_keys()) out.push_back(at(k));
    return out;
}

std::vector<double> LuaValue::numbers() const {
    std::vector<double> out;
    for (auto& v : sequence()) out.push_back(v.number());
    return out;
}

std::vector<int> LuaValue::ints() const {
    std::vector<int> out;
    for (auto& v : sequence()) out.push_back((int)v.number());
    return out;
}

LuaValue read_lua_string(const std::string& text) {
    Lexer lx(text);
    Parser p(lx.run());
    return p.chunk();
}

LuaValue read_lua_file(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return read_lua_string(ss.str());
}

}  // namespace gdtk
