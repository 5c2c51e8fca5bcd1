// Minimal stand-in for the TCLAP command-line library (the reference's
// deps/tclap submodule is empty in this tree).  Provides only what the
// reference's fluidtest uses (test/src/main.cpp:81-107, 152-156):
// CmdLine(message, delimiter, version), ValueArg<T>(flag, name, desc,
// required, default, typeDesc), CmdLine::add, CmdLine::parse,
// ValueArg::getValue and ArgException::error / argId.  Accepts "-f value"
// and "--name value".  Used only to compile the reference's fluidtest
// against this repository's FluidSystem drop-in.
#ifndef SPH_REF_TCLAP_CMDLINE_H
#define SPH_REF_TCLAP_CMDLINE_H

#include <cstdlib>
#include <exception>
#include <sstream>
#include <string>
#include <vector>

namespace TCLAP {

class ArgException : public std::exception {
public:
    ArgException(const std::string& msg, const std::string& id) : msg_(msg), id_(id) {}
    std::string error() const { return msg_; }
    std::string argId() const { return id_; }
    const char* what() const noexcept override { return msg_.c_str(); }

private:
    std::string msg_, id_;
};

class Arg {
public:
    Arg(const std::string& flag, const std::string& name, bool req) : flag_(flag), name_(name), req_(req) {}
    virtual ~Arg() {}
    bool matches(const std::string& a) const { return a == "-" + flag_ || a == "--" + name_; }
    virtual void set(const std::string& v) = 0;
    bool required() const { return req_; }
    bool seen() const { return seen_; }
    const std::string& name() const { return name_; }

protected:
    std::string flag_, name_;
    bool req_;
    bool seen_ = false;
};

template <class T>
class ValueArg : public Arg {
public:
    ValueArg(const std::string& flag, const std::string& name, const std::string& /*desc*/, bool req, T value,
             const std::string& /*typeDesc*/)
        : Arg(flag, name, req), value_(value) {}
    void set(const std::string& v) override {
        std::istringstream is(v);
        T t;
        if (!(is >> t)) throw ArgException("Couldn't read argument value from string '" + v + "'", name_);
        value_ = t;
        seen_ = true;
    }
    const T& getValue() const { return value_; }

private:
    T value_;
};

template <>
inline void ValueArg<std::string>::set(const std::string& v) {
    value_ = v;
    seen_ = true;
}

class CmdLine {
public:
    CmdLine(const std::string& /*message*/, char /*delimiter*/ = ' ', const std::string& /*version*/ = "none") {}
    void add(Arg& a) { args_.push_back(&a); }
    void parse(int argc, const char* const* argv) {
        for (int i = 1; i < argc; ++i) {
            const std::string a = argv[i];
            bool hit = false;
            for (Arg* arg : args_) {
                if (!arg->matches(a)) continue;
                if (i + 1 >= argc) throw ArgException("Missing a value for this argument!", arg->name());
                arg->set(argv[++i]);
                hit = true;
                break;
            }
            if (!hit) throw ArgException("Couldn't find match for argument", a);
        }
        for (Arg* arg : args_)
            if (arg->required() && !arg->seen()) throw ArgException("Required argument missing", arg->name());
    }

private:
    std::vector<Arg*> args_;
};

}  // namespace TCLAP

#endif
