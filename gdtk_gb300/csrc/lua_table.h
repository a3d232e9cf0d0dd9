// lua_table.h -- reader for the Lua data files written by gdtk's prep-gas and prep-chem.
//
// Those files (read by the reference with a full Lua interpreter: gas/composite_gas.d:37-120,
// kinetics/chemistry_update.d:42-137) are chunks of assignment statements whose right-hand
// sides are literals and table constructors, e.g.
//     species = {[0]='N2', [1]='O2', }
//     db['N2'].thermoCoeffs = { nsegments = 3, T_break_points = {200.0, 1000.0, 6000.0, 20000.0}, ... }
//     reaction[1] = { type = "elementary", frc = {model='Arrhenius', A=7.0e15, n=-1.6, C=1.132e5}, ... }
// This reader accepts exactly that subset: statements `name{.field|[expr]} = expr`, numbers,
// strings, booleans, nil, unary minus and table constructors.  Anything else is an error.
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gdtk {

struct LuaValue;
using LuaTablePtr = std::shared_ptr<std::map<std::string, LuaValue>>;

// Table keys are stored as strings: a number key k is stored as "#k" (integer-valued numbers
// only), a string key s as s.  Lua's implicit array part of a constructor is numbered from 1.
struct LuaValue {
    enum Kind { NIL, BOOL, NUMBER, STRING, TABLE } kind = NIL;
    bool b = false;
    double num = 0.0;
    std::string str;
    LuaTablePtr tab;

    bool is_nil() const { return kind == NIL; }
    double number() const {
        if (kind != NUMBER) throw std::runtime_error("Lua value is not a number");
        return num;
    }
    const std::string& string() const {
        if (kind != STRING) throw std::runtime_error("Lua value is not a string");
        return str;
    }
    bool boolean() const {
        if (kind == BOOL) return b;
        return kind != NIL;
    }
    const LuaValue& get(const std::string& key) const;   // NIL value if absent
    const LuaValue& at(long index) const;                 // integer key
    bool has(const std::string& key) const { return !get(key).is_nil(); }
    // Values of integer keys in ascending key order (a Lua sequence, from [0] or [1]).
    std::vector<LuaValue> sequence() const;
    std::vector<double> numbers() const;
    std::vector<int> ints() const;
    // Integer keys present, ascending.
    std::vector<long> int_keys() const;
};

// Parses a whole file; returns the table of globals it assigns.
LuaValue read_lua_file(const std::string& path);
LuaValue read_lua_string(const std::string& text);

}  // namespace gdtk
