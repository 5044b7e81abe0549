// A project-written subset of the Boost.ProgramOptions 1.x API: the classes
// and functions the reference's configuration layer names
// (core/src/include/Configured.hpp:115-181, core/src/Configurator.cpp:14-50,
// core/src/CommandLineParser.cpp:34-60, core/src/include/EnumWrapper.hpp:100-112),
// written from the library's documented interface so that the reference's
// module headers compile and link where Boost is not installed.
//
// TEST INFRASTRUCTURE ONLY (oracle/).  Behaviour kept: options declared with
// add_options()(name, value<T>()->default_value(d), description); "--name=v"
// and "--name v" on the command line; "[section]" and "key = value" lines in a
// configuration stream, giving "section.key"; store() keeps the first value
// stored for a name and fills declared defaults for names not given;
// variables_map[name].as<T>(); unregistered names are skipped when allowed and
// are an error otherwise.  Values are parsed by operator>> (std::string: the
// whole token; bool: true/false/1/0/yes/no/on/off), or by a validate()
// overload found by argument-dependent lookup, as the library does for user
// types.  Not kept: positional options, short-option bundling, help layout.
#pragma once

#include <algorithm>
#include <any>
#include <cctype>
#include <istream>
#include <map>
#include <memory>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace boost {

using std::any;
using std::any_cast;

namespace program_options {

class error : public std::logic_error {
public:
    explicit error(const std::string& what)
        : std::logic_error(what)
    {
    }
};

class unknown_option : public error {
public:
    explicit unknown_option(const std::string& name)
        : error("unrecognised option '" + name + "'")
    {
    }
};

class validation_error : public error {
public:
    enum kind_t {
        multiple_values_not_allowed = 30,
        at_least_one_value_required,
        invalid_bool_value,
        invalid_option_value,
        invalid_option
    };
    explicit validation_error(kind_t kind, const std::string& option_name = "",
        const std::string& original_token = "")
        : error(message(kind, option_name, original_token))
        , m_kind(kind)
    {
    }
    kind_t kind() const { return m_kind; }

private:
    static std::string message(kind_t k, const std::string& name, const std::string& token)
    {
        std::string s;
        switch (k) {
        case multiple_values_not_allowed: s = "multiple values not allowed"; break;
        case at_least_one_value_required: s = "at least one value required"; break;
        case invalid_bool_value: s = "invalid boolean value"; break;
        case invalid_option_value: s = "invalid option value"; break;
        default: s = "invalid option"; break;
        }
        if (!name.empty())
            s += " for '" + name + "'";
        if (!token.empty())
            s += ": '" + token + "'";
        return s;
    }
    kind_t m_kind;
};

namespace validators {
    inline void check_first_occurrence(const std::any& v)
    {
        if (v.has_value())
            throw validation_error(validation_error::multiple_values_not_allowed);
    }
    inline const std::string& get_single_string(const std::vector<std::string>& v, bool allow_empty = false)
    {
        static const std::string empty;
        if (v.size() > 1)
            throw validation_error(validation_error::multiple_values_not_allowed);
        if (v.empty()) {
            if (!allow_empty)
                throw validation_error(validation_error::at_least_one_value_required);
            return empty;
        }
        return v.front();
    }
}

namespace detail {
    inline std::string trim(const std::string& s)
    {
        size_t a = 0, b = s.size();
        while (a < b && std::isspace(static_cast<unsigned char>(s[a])))
            ++a;
        while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1])))
            --b;
        return s.substr(a, b - a);
    }

    template <class T> struct is_vector : std::false_type { };
    template <class U, class A> struct is_vector<std::vector<U, A>> : std::true_type {
        using element = U;
    };

    template <class T> T parse_scalar(const std::string& token)
    {
        if constexpr (std::is_same_v<T, std::string>) {
            return token;
        } else if constexpr (std::is_same_v<T, bool>) {
            std::string t = trim(token);
            std::transform(t.begin(), t.end(), t.begin(), [](unsigned char c) { return std::tolower(c); });
            if (t.empty() || t == "true" || t == "1" || t == "yes" || t == "on")
                return true;
            if (t == "false" || t == "0" || t == "no" || t == "off")
                return false;
            throw validation_error(validation_error::invalid_bool_value, "", token);
        } else {
            std::istringstream is(token);
            T v {};
            is >> v;
            if (is.fail())
                throw validation_error(validation_error::invalid_option_value, "", token);
            is >> std::ws;
            if (!is.eof())
                throw validation_error(validation_error::invalid_option_value, "", token);
            return v;
        }
    }

    // the library's customisation point: a user type T supplies
    // void validate(boost::any&, const std::vector<std::string>&, T*, int)
    // in its own namespace; this overload is the fallback
    template <class T> void validate(std::any& v, const std::vector<std::string>& tokens, T*, long)
    {
        if constexpr (is_vector<T>::value) {
            using E = typename is_vector<T>::element;
            T out = v.has_value() ? std::any_cast<T>(v) : T {};
            for (const auto& t : tokens)
                out.push_back(parse_scalar<E>(t));
            v = out;
        } else {
            validators::check_first_occurrence(v);
            v = parse_scalar<T>(validators::get_single_string(tokens, std::is_same_v<T, bool>));
        }
    }

    template <class T> std::any parse_value(const std::vector<std::string>& tokens)
    {
        std::any v;
        validate(v, tokens, static_cast<T*>(nullptr), 0);
        return v;
    }
}

class value_semantic {
public:
    virtual ~value_semantic() = default;
    virtual bool apply_default(std::any& v) const = 0;
    virtual std::any parse(const std::vector<std::string>& tokens) const = 0;
    virtual bool is_multitoken() const { return false; }
    virtual bool takes_value() const { return true; }
};

template <class T> class typed_value : public value_semantic {
public:
    typed_value* default_value(const T& v)
    {
        m_default = v;
        return this;
    }
    typed_value* default_value(const T& v, const std::string&) { return default_value(v); }
    typed_value* implicit_value(const T& v)
    {
        m_implicit = v;
        return this;
    }
    typed_value* multitoken()
    {
        m_multi = true;
        return this;
    }
    typed_value* composing() { return this; }
    typed_value* required() { return this; }
    typed_value* value_name(const std::string&) { return this; }

    bool apply_default(std::any& v) const override
    {
        if (!m_default.has_value())
            return false;
        v = m_default;
        return true;
    }
    std::any parse(const std::vector<std::string>& tokens) const override
    {
        if (tokens.empty() && m_implicit.has_value())
            return m_implicit;
        return detail::parse_value<T>(tokens);
    }
    bool is_multitoken() const override { return m_multi; }

private:
    std::any m_default;
    std::any m_implicit;
    bool m_multi = false;
};

template <class T> typed_value<T>* value() { return new typed_value<T>(); }
template <class T> typed_value<T>* value(T*) { return new typed_value<T>(); }

class untyped_value : public value_semantic {
public:
    bool apply_default(std::any&) const override { return false; }
    std::any parse(const std::vector<std::string>&) const override { return std::any(true); }
    bool takes_value() const override { return false; }
};

class option_description {
public:
    option_description(const std::string& names, const value_semantic* s, const std::string& description)
        : m_sem(s)
        , m_description(description)
    {
        const size_t comma = names.find(',');
        m_long = names.substr(0, comma);
        if (comma != std::string::npos)
            m_short = names.substr(comma + 1);
    }
    const std::string& long_name() const { return m_long; }
    const std::string& short_name() const { return m_short; }
    const std::string& description() const { return m_description; }
    std::shared_ptr<const value_semantic> semantic() const { return m_sem; }

private:
    std::string m_long, m_short;
    std::shared_ptr<const value_semantic> m_sem;
    std::string m_description;
};

class options_description;

class options_description_easy_init {
public:
    explicit options_description_easy_init(options_description* owner)
        : m_owner(owner)
    {
    }
    options_description_easy_init& operator()(const char* name, const char* description);
    options_description_easy_init& operator()(const char* name, const value_semantic* s);
    options_description_easy_init& operator()(const char* name, const value_semantic* s, const char* description);

private:
    options_description* m_owner;
};

class options_description {
public:
    static const unsigned m_default_line_length = 80;

    options_description(unsigned = m_default_line_length, unsigned = m_default_line_length / 2) { }
    explicit options_description(const std::string& caption, unsigned = m_default_line_length,
        unsigned = m_default_line_length / 2)
        : m_caption(caption)
    {
    }

    options_description_easy_init add_options() { return options_description_easy_init(this); }
    void add(std::shared_ptr<option_description> d) { m_options.push_back(std::move(d)); }
    options_description& add(const options_description& other)
    {
        m_options.insert(m_options.end(), other.m_options.begin(), other.m_options.end());
        return *this;
    }
    const option_description* find_nothrow(const std::string& name, bool = false, bool = false,
        bool = false) const
    {
        for (const auto& o : m_options)
            if (o->long_name() == name || (!o->short_name().empty() && o->short_name() == name))
                return o.get();
        return nullptr;
    }
    const option_description& find(const std::string& name, bool approx = false) const
    {
        const option_description* d = find_nothrow(name, approx);
        if (!d)
            throw unknown_option(name);
        return *d;
    }
    const std::vector<std::shared_ptr<option_description>>& options() const { return m_options; }

    friend std::ostream& operator<<(std::ostream& os, const options_description& d)
    {
        if (!d.m_caption.empty())
            os << d.m_caption << "\n";
        for (const auto& o : d.m_options)
            os << "  --" << o->long_name() << "  " << o->description() << "\n";
        return os;
    }

private:
    std::string m_caption;
    std::vector<std::shared_ptr<option_description>> m_options;
};

inline options_description_easy_init& options_description_easy_init::operator()(
    const char* name, const char* description)
{
    m_owner->add(std::make_shared<option_description>(name, new untyped_value(), description));
    return *this;
}
inline options_description_easy_init& options_description_easy_init::operator()(
    const char* name, const value_semantic* s)
{
    m_owner->add(std::make_shared<option_description>(name, s, ""));
    return *this;
}
inline options_description_easy_init& options_description_easy_init::operator()(
    const char* name, const value_semantic* s, const char* description)
{
    m_owner->add(std::make_shared<option_description>(name, s, description));
    return *this;
}

class variable_value {
public:
    variable_value() = default;
    variable_value(const std::any& v, bool defaulted)
        : m_value(v)
        , m_defaulted(defaulted)
    {
    }
    template <class T> const T& as() const { return std::any_cast<const T&>(m_value); }
    template <class T> T& as() { return std::any_cast<T&>(m_value); }
    bool empty() const { return !m_value.has_value(); }
    bool defaulted() const { return m_defaulted; }
    const std::any& value() const { return m_value; }
    std::any& value() { return m_value; }

private:
    std::any m_value;
    bool m_defaulted = false;
};

class variables_map : public std::map<std::string, variable_value> {
public:
    const variable_value& operator[](const std::string& name) const
    {
        static const variable_value empty;
        auto it = find(name);
        return it == end() ? empty : it->second;
    }
};

template <class Char> class basic_option {
public:
    std::string string_key;
    std::vector<std::string> value;
    bool unregistered = false;
};
using option = basic_option<char>;

template <class Char> class basic_parsed_options {
public:
    explicit basic_parsed_options(const options_description* d)
        : description(d)
    {
    }
    std::vector<basic_option<Char>> options;
    const options_description* description;
};
using parsed_options = basic_parsed_options<char>;

namespace command_line_style {
    enum style_t {
        allow_long = 1,
        allow_short = allow_long << 1,
        allow_dash_for_short = allow_short << 1,
        allow_slash_for_short = allow_dash_for_short << 1,
        long_allow_adjacent = allow_slash_for_short << 1,
        long_allow_next = long_allow_adjacent << 1,
        short_allow_adjacent = long_allow_next << 1,
        short_allow_next = short_allow_adjacent << 1,
        allow_sticky = short_allow_next << 1,
        allow_guessing = allow_sticky << 1,
        long_case_insensitive = allow_guessing << 1,
        short_case_insensitive = long_case_insensitive << 1,
        case_insensitive = (long_case_insensitive | short_case_insensitive),
        allow_long_disguise = short_case_insensitive << 1,
        unix_style = (allow_short | short_allow_adjacent | short_allow_next | allow_long | long_allow_adjacent
            | long_allow_next | allow_sticky | allow_guessing | allow_dash_for_short),
        default_style = unix_style
    };
}

template <class Char> class basic_command_line_parser {
public:
    basic_command_line_parser(int argc, const Char* const argv[])
    {
        for (int i = 1; i < argc; ++i)
            m_args.emplace_back(argv[i]);
    }
    basic_command_line_parser(const std::vector<std::string>& args)
        : m_args(args)
    {
    }
    basic_command_line_parser& options(const options_description& d)
    {
        m_desc = &d;
        return *this;
    }
    basic_command_line_parser& style(int) { return *this; }
    basic_command_line_parser& allow_unregistered()
    {
        m_allowUnregistered = true;
        return *this;
    }

    basic_parsed_options<Char> run() const
    {
        basic_parsed_options<Char> out(m_desc);
        for (size_t i = 0; i < m_args.size(); ++i) {
            const std::string& a = m_args[i];
            if (a.size() < 2 || a[0] != '-') {
                if (!m_allowUnregistered)
                    throw error("positional argument '" + a + "' not allowed");
                continue;
            }
            std::string key = a.substr(a[1] == '-' ? 2 : 1);
            std::vector<std::string> vals;
            const size_t eq = key.find('=');
            bool inlineValue = eq != std::string::npos;
            if (inlineValue) {
                vals.push_back(key.substr(eq + 1));
                key = key.substr(0, eq);
            }
            const option_description* d = m_desc ? m_desc->find_nothrow(key) : nullptr;
            if (!d) {
                if (!m_allowUnregistered)
                    throw unknown_option(key);
                continue;
            }
            const auto sem = d->semantic();
            if (!inlineValue && sem->takes_value()) {
                while (i + 1 < m_args.size() && !(m_args[i + 1].size() > 1 && m_args[i + 1][0] == '-')) {
                    vals.push_back(m_args[++i]);
                    if (!sem->is_multitoken())
                        break;
                }
            }
            basic_option<Char> o;
            o.string_key = d->long_name();
            o.value = vals;
            out.options.push_back(o);
        }
        return out;
    }

private:
    std::vector<std::string> m_args;
    const options_description* m_desc = nullptr;
    bool m_allowUnregistered = false;
};
using command_line_parser = basic_command_line_parser<char>;

inline parsed_options parse_command_line(int argc, const char* const argv[], const options_description& d,
    int = command_line_style::default_style)
{
    return command_line_parser(argc, argv).options(d).run();
}

inline parsed_options parse_config_file(std::istream& is, const options_description& d,
    bool allow_unregistered = false)
{
    parsed_options out(&d);
    std::string line, prefix;
    while (std::getline(is, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos)
            line.erase(hash);
        line = detail::trim(line);
        if (line.empty())
            continue;
        if (line.front() == '[' && line.back() == ']') {
            prefix = detail::trim(line.substr(1, line.size() - 2));
            if (!prefix.empty())
                prefix += ".";
            continue;
        }
        const size_t eq = line.find('=');
        if (eq == std::string::npos)
            throw error("the configuration line '" + line + "' has no '='");
        const std::string key = prefix + detail::trim(line.substr(0, eq));
        const std::string val = detail::trim(line.substr(eq + 1));
        if (!d.find_nothrow(key)) {
            if (!allow_unregistered)
                throw unknown_option(key);
            continue;
        }
        option o;
        o.string_key = key;
        o.value.push_back(val);
        out.options.push_back(o);
    }
    return out;
}

// The first value stored for a name is kept (a later store does not change
// it unless it was a default); declared defaults fill the names not given.
inline void store(const parsed_options& p, variables_map& vm)
{
    std::map<std::string, std::vector<std::string>> tokens;
    std::vector<std::string> order;
    for (const auto& o : p.options) {
        auto it = tokens.find(o.string_key);
        if (it == tokens.end()) {
            order.push_back(o.string_key);
            tokens[o.string_key] = o.value;
        } else {
            it->second.insert(it->second.end(), o.value.begin(), o.value.end());
        }
    }
    for (const auto& key : order) {
        auto have = vm.find(key);
        if (have != vm.end() && !have->second.defaulted())
            continue;
        const option_description* d = p.description ? p.description->find_nothrow(key) : nullptr;
        if (!d)
            continue;
        try {
            vm.insert_or_assign(key, variable_value(d->semantic()->parse(tokens[key]), false));
        } catch (const validation_error& e) {
            throw validation_error(e.kind(), key, tokens[key].empty() ? "" : tokens[key].front());
        }
    }
    if (p.description) {
        for (const auto& o : p.description->options()) {
            if (vm.count(o->long_name()))
                continue;
            std::any v;
            if (o->semantic()->apply_default(v))
                vm.emplace(o->long_name(), variable_value(v, true));
        }
    }
}

inline void notify(variables_map&) { }

}
}
