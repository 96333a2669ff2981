#include "json.h"

#include <cctype>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <sstream>

namespace bt::json {

NodeP Node::find(const std::string &key) const
{
    if(kind != Kind::Group)
        return nullptr;
    for(auto &m : members)
        if(m.first == key)
            return m.second;
    return nullptr;
}

NodeP Node::child(const std::string &key) const
{
    if(kind != Kind::Group)
        throw ParseError("group node expected when looking up '" + key + "'");
    auto r = find(key);
    if(!r)
        throw ParseError("missing child node '" + key + "'");
    return r;
}

namespace {

class Lexer
{
public:
    explicit Lexer(const std::string &t) : s_(t) {}

    NodeP parse_document()
    {
        skip_ws();
        NodeP n = parse_value();
        skip_ws();
        if(i_ != s_.size())
            fail("trailing characters after JSON document");
        return n;
    }

private:
    const std::string &s_;
    size_t i_ = 0;

    [[noreturn]] void fail(const std::string &msg)
    {
        size_t line = 1;
        for(size_t k = 0; k < i_ && k < s_.size(); ++k)
            if(s_[k] == '\n')
                ++line;
        throw ParseError("json: " + msg + " (line " + std::to_string(line) + ")");
    }

    void skip_ws()
    {
        for(;;)
        {
            while(i_ < s_.size() && std::isspace((unsigned char)s_[i_]))
                ++i_;
            if(i_ + 1 < s_.size() && s_[i_] == '/' && s_[i_ + 1] == '/')
            {
                while(i_ < s_.size() && s_[i_] != '\n')
                    ++i_;
                continue;
            }
            if(i_ + 1 < s_.size() && s_[i_] == '/' && s_[i_ + 1] == '*')
            {
                size_t e = s_.find("*/", i_ + 2);
                if(e == std::string::npos)
                    fail("unterminated comment");
                i_ = e + 2;
                continue;
            }
            break;
        }
    }

    NodeP parse_value()
    {
        if(i_ >= s_.size())
            fail("unexpected end of input");
        char c = s_[i_];
        if(c == '{')
            return parse_object();
        if(c == '[')
            return parse_array();
        auto v = std::make_shared<Node>();
        v->kind = Node::Kind::Value;
        if(c == '"')
        {
            v->str = parse_string();
            return v;
        }
        if(s_.compare(i_, 4, "true") == 0)
        {
            i_ += 4;
            v->str = "true";
            return v;
        }
        if(s_.compare(i_, 5, "false") == 0)
        {
            i_ += 5;
            v->str = "false";
            return v;
        }
        if(s_.compare(i_, 4, "null") == 0)
        {
            i_ += 4;
            v->str = "";
            return v;
        }
        if(c == '-' || std::isdigit((unsigned char)c))
        {
            size_t b = i_;
            bool is_float = false;
            if(s_[i_] == '-')
                ++i_;
            while(i_ < s_.size())
            {
                char d = s_[i_];
                if(std::isdigit((unsigned char)d))
                    ++i_;
                else if(d == '.' || d == 'e' || d == 'E' || d == '+' || d == '-')
                {
                    is_float = true;
                    ++i_;
                }
                else
                    break;
            }
            const std::string num = s_.substr(b, i_ - b);
            char *end = nullptr;
            if(is_float)
            {
                const double d = std::strtod(num.c_str(), &end);
                if(end != num.c_str() + num.size())
                    fail("bad number '" + num + "'");
                v->str = std::to_string(static_cast<float>(d));
            }
            else
            {
                const long long ll = std::strtoll(num.c_str(), &end, 10);
                if(end != num.c_str() + num.size())
                    fail("bad number '" + num + "'");
                v->str = std::to_string(static_cast<int>(ll));
            }
            return v;
        }
        fail(std::string("unexpected character '") + c + "'");
    }

    std::string parse_string()
    {
        ++i_;  // opening quote
        std::string out;
        while(i_ < s_.size() && s_[i_] != '"')
        {
            char c = s_[i_++];
            if(c == '\\')
            {
                if(i_ >= s_.size())
                    fail("bad escape");
                char e = s_[i_++];
                switch(e)
                {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u':
                {
                    if(i_ + 4 > s_.size())
                        fail("bad unicode escape");
                    unsigned cp = (unsigned)std::strtoul(s_.substr(i_, 4).c_str(), nullptr, 16);
                    i_ += 4;
                    if(cp < 0x80)
                        out += (char)cp;
                    else if(cp < 0x800)
                    {
                        out += (char)(0xc0 | (cp >> 6));
                        out += (char)(0x80 | (cp & 0x3f));
                    }
                    else
                    {
                        out += (char)(0xe0 | (cp >> 12));
                        out += (char)(0x80 | ((cp >> 6) & 0x3f));
                        out += (char)(0x80 | (cp & 0x3f));
                    }
                    break;
                }
                default: out += e; break;
                }
            }
            else
                out += c;
        }
        if(i_ >= s_.size())
            fail("unterminated string");
        ++i_;
        return out;
    }

    NodeP parse_object()
    {
        ++i_;
        auto g = std::make_shared<Node>();
        g->kind = Node::Kind::Group;
        skip_ws();
        if(i_ < s_.size() && s_[i_] == '}')
        {
            ++i_;
            return g;
        }
        for(;;)
        {
            skip_ws();
            if(i_ >= s_.size() || s_[i_] != '"')
                fail("object key expected");
            std::string key = parse_string();
            skip_ws();
            if(i_ >= s_.size() || s_[i_] != ':')
                fail("':' expected");
            ++i_;
            skip_ws();
            NodeP v = parse_value();
            bool replaced = false;
            for(auto &m : g->members)
                if(m.first == key)
                {
                    m.second = v;
                    replaced = true;
                }
            if(!replaced)
                g->members.emplace_back(std::move(key), std::move(v));
            skip_ws();
            if(i_ < s_.size() && s_[i_] == ',')
            {
                ++i_;
                continue;
            }
            if(i_ < s_.size() && s_[i_] == '}')
            {
                ++i_;
                return g;
            }
            fail("',' or '}' expected");
        }
    }

    NodeP parse_array()
    {
        ++i_;
        auto a = std::make_shared<Node>();
        a->kind = Node::Kind::Array;
        skip_ws();
        if(i_ < s_.size() && s_[i_] == ']')
        {
            ++i_;
            return a;
        }
        for(;;)
        {
            skip_ws();
            a->elems.push_back(parse_value());
            skip_ws();
            if(i_ < s_.size() && s_[i_] == ',')
            {
                ++i_;
                continue;
            }
            if(i_ < s_.size() && s_[i_] == ']')
            {
                ++i_;
                return a;
            }
            fail("',' or ']' expected");
        }
    }
};

std::string read_file(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if(!f)
        throw ParseError("cannot open file '" + path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::vector<std::string> split_path(const std::string &p)
{
    std::vector<std::string> out;
    std::string cur;
    for(char c : p)
    {
        if(c == '/')
        {
            if(!cur.empty())
                out.push_back(cur);
            cur.clear();
        }
        else
            cur += c;
    }
    if(!cur.empty())
        out.push_back(cur);
    return out;
}

bool parse_index(const std::string &s, size_t &idx)
{
    if(s.empty())
        return false;
    for(char c : s)
        if(!std::isdigit((unsigned char)c))
            return false;
    idx = std::strtoul(s.c_str(), nullptr, 10);
    return true;
}

// Resolve "a/b/c": the first section is looked up from the innermost enclosing node
// outwards ("$root" starts at the document root), then the rest walks down.
NodeP find_node(const std::vector<NodeP> &path, const std::string &ref)
{
    const auto secs = split_path(ref);
    if(secs.empty())
        throw ParseError("invalid node path: " + ref);
    int start = -1;
    if(secs[0] == "$root")
        start = 0;
    else
    {
        for(int k = static_cast<int>(path.size()) - 1; k >= 0; --k)
        {
            const NodeP &n = path[k];
            size_t idx;
            if(n->is_group() && n->find(secs[0]))
            {
                start = k;
                break;
            }
            if(n->is_array() && parse_index(secs[0], idx) && idx < n->elems.size())
            {
                start = k;
                break;
            }
        }
    }
    if(start < 0)
        throw ParseError("invalid node path: " + ref);
    NodeP node = path[start];
    for(size_t i = 0; i < secs.size(); ++i)
    {
        if(i == 0 && secs[i] == "$root")
            continue;
        size_t idx;
        if(node->is_group())
        {
            node = node->find(secs[i]);
            if(!node)
                throw ParseError("invalid node path: " + ref);
        }
        else if(node->is_array() && parse_index(secs[i], idx) && idx < node->elems.size())
            node = node->elems[idx];
        else
            throw ParseError("invalid node path: " + ref);
    }
    return node;
}

void resolve_references(std::vector<NodeP> &path, NodeP &node)
{
    if(node->is_group())
    {
        path.push_back(node);
        for(auto &m : node->members)
            resolve_references(path, m.second);
        path.pop_back();
    }
    else if(node->is_array())
    {
        path.push_back(node);
        for(auto &e : node->elems)
            resolve_references(path, e);
        path.pop_back();
    }
    else if(node->str.rfind("$reference{", 0) == 0)
    {
        if(node->str.back() != '}')
            throw ParseError("'}' for '$reference{' is not found");
        const std::string p = node->str.substr(11, node->str.size() - 12);
        node = find_node(path, p);
    }
}

} // namespace

NodeP parse_text(const std::string &text)
{
    Lexer lx(text);
    return lx.parse_document();
}

NodeP parse_scene_text(std::string src, const std::string &include_dir)
{
    for(int guard = 0;; ++guard)
    {
        if(guard > 10000)
            throw ParseError("too many $include directives (recursive include?)");
        size_t beg = src.find("\"$include{");
        if(beg == std::string::npos)
            break;
        size_t name_beg = beg + 10;
        size_t end = src.find("}\"", name_beg);
        if(end == std::string::npos)
            throw ParseError("failed to find the enclosing '}' of a '$include{'");
        std::filesystem::path inc = src.substr(name_beg, end - name_beg);
        if(inc.is_relative())
            inc = std::filesystem::path(include_dir) / inc;
        if(!std::filesystem::exists(inc))
            throw ParseError("included file '" + inc.string() + "' is not found");
        src = src.substr(0, beg) + read_file(inc.lexically_normal().string()) + src.substr(end + 2);
    }
    NodeP root = parse_text(src);
    if(!root->is_group())
        throw ParseError("root node is not a group");
    std::vector<NodeP> path = { root };
    for(auto &m : root->members)
        resolve_references(path, m.second);
    return root;
}

NodeP parse_scene_file(const std::string &path, const std::string &include_dir)
{
    return parse_scene_text(read_file(path), include_dir);
}

float as_float(const NodeP &n)
{
    if(!n || !n->is_value())
        throw ParseError("scalar value expected");
    try { return std::stof(n->str); }
    catch(...) { throw ParseError("cannot parse float from '" + n->str + "'"); }
}

int as_int(const NodeP &n)
{
    if(!n || !n->is_value())
        throw ParseError("scalar value expected");
    try { return std::stoi(n->str); }
    catch(...) { throw ParseError("cannot parse int from '" + n->str + "'"); }
}

bool as_bool(const NodeP &n)
{
    if(!n || !n->is_value())
        throw ParseError("scalar value expected");
    return n->str == "true";
}

std::string as_string(const NodeP &n)
{
    if(!n || !n->is_value())
        throw ParseError("string value expected");
    return n->str;
}

V3 as_vec3(const NodeP &n)
{
    if(n->is_array())
    {
        if(n->elems.size() == 1)
            return V3(as_float(n->elems[0]));
        if(n->elems.size() == 3)
            return V3(as_float(n->elems[0]), as_float(n->elems[1]), as_float(n->elems[2]));
        throw ParseError("unexpected array size: " + std::to_string(n->elems.size()));
    }
    if(n->is_value())
        return V3(as_float(n));
    throw ParseError("unexpected group node");
}

V3 as_spectrum(const NodeP &n) { return as_vec3(n); }

float as_degree(const NodeP &n)
{
    if(!n->is_group())
        throw ParseError("group expected");
    if(auto c = n->find("deg"))
        return as_float(c);
    if(auto c = n->find("rad"))
        return 180.0f / PI * as_float(c);
    throw ParseError("invalid angle node");
}

float as_radian(const NodeP &n)
{
    if(!n->is_group())
        throw ParseError("group expected");
    if(auto c = n->find("deg"))
        return PI / 180.0f * as_float(c);
    if(auto c = n->find("rad"))
        return as_float(c);
    throw ParseError("invalid angle node");
}

float float_or(const NodeP &p, const std::string &k, float d)
{
    auto n = p ? p->find(k) : nullptr;
    return n ? as_float(n) : d;
}

int int_or(const NodeP &p, const std::string &k, int d)
{
    auto n = p ? p->find(k) : nullptr;
    return n ? as_int(n) : d;
}

bool bool_or(const NodeP &p, const std::string &k, bool d)
{
    auto n = p ? p->find(k) : nullptr;
    return n ? as_bool(n) : d;
}

} // namespace bt::json
