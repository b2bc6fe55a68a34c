// Loader for a GP19 bremsstrahlung table in the reference's header format.
//
// The reference compiles its table in (GP19Table.hpp, included by
// kernel_brem_GP19.hpp): integer constants GP19_nb_dims, GP19_Ye_dims,
// GP19_T_dims, GP19_w_dims and arrays GP19_nb_axis, GP19_lognb_axis,
// GP19_Ye_axis, GP19_T_axis, GP19_w_axis, GP19_logw_axis and GP19_data
// (flat [nb][Ye][T][w], kernel_brem_GP19.hpp:101-102).  This file reads such a
// header as text at run time and hands the arrays to bnsn_gp19_set_table, so
// a user who has the published table can load it without rebuilding.  The
// log axes are optional (computed from the linear ones when absent); nested
// braces, comments and numeric suffixes (f, L) in the initialisers are
// accepted.

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bns_nurates_gb300.h"

namespace {

bool ident_char(char c) { return std::isalnum((unsigned char)c) || c == '_'; }

// Position after the '=' of the declaration of `name` (npos if absent):
// an occurrence of the identifier followed by an optional [...] and '='.
size_t find_decl(const std::string& s, const char* name)
{
    const size_t len = strlen(name);
    for (size_t pos = s.find(name); pos != std::string::npos; pos = s.find(name, pos + 1))
    {
        if (pos > 0 && ident_char(s[pos - 1]))
            continue;
        size_t q = pos + len;
        if (q < s.size() && ident_char(s[q]))
            continue;
        while (q < s.size() && std::isspace((unsigned char)s[q]))
            ++q;
        if (q < s.size() && s[q] == '[')
        {
            const size_t close = s.find(']', q);
            if (close == std::string::npos)
                return std::string::npos;
            q = close + 1;
            while (q < s.size() && std::isspace((unsigned char)s[q]))
                ++q;
        }
        if (q < s.size() && s[q] == '=' && (q + 1 >= s.size() || s[q + 1] != '='))
            return q + 1;
    }
    return std::string::npos;
}

// Skips whitespace and comments.
size_t skip_blank(const std::string& s, size_t q)
{
    while (q < s.size())
    {
        if (std::isspace((unsigned char)s[q]))
            ++q;
        else if (s.compare(q, 2, "//") == 0)
        {
            const size_t e = s.find('\n', q);
            q = e == std::string::npos ? s.size() : e + 1;
        }
        else if (s.compare(q, 2, "/*") == 0)
        {
            const size_t e = s.find("*/", q + 2);
            q = e == std::string::npos ? s.size() : e + 2;
        }
        else
            break;
    }
    return q;
}

bool read_int(const std::string& s, const char* name, int* out)
{
    size_t q = find_decl(s, name);
    if (q == std::string::npos)
        return false;
    q = skip_blank(s, q);
    char* end      = nullptr;
    const long val = strtol(s.c_str() + q, &end, 10);
    if (end == s.c_str() + q)
        return false;
    *out = (int)val;
    return true;
}

// Numbers of the brace initialiser of `name` (nested braces flattened).
bool read_array(const std::string& s, const char* name, std::vector<double>* out)
{
    size_t q = find_decl(s, name);
    if (q == std::string::npos)
        return false;
    q = skip_blank(s, q);
    if (q >= s.size() || s[q] != '{')
        return false;
    int depth = 0;
    out->clear();
    while (q < s.size())
    {
        q = skip_blank(s, q);
        if (q >= s.size())
            return false;
        const char c = s[q];
        if (c == '{')
        {
            ++depth;
            ++q;
        }
        else if (c == '}')
        {
            ++q;
            if (--depth == 0)
                return true;
        }
        else if (c == ',')
            ++q;
        else
        {
            char* end      = nullptr;
            const double v = strtod(s.c_str() + q, &end);
            if (end == s.c_str() + q)
                return false;
            out->push_back(v);
            q = (size_t)(end - s.c_str());
            while (q < s.size() && (s[q] == 'f' || s[q] == 'F' || s[q] == 'l' || s[q] == 'L'))
                ++q;
        }
    }
    return false;
}

} // namespace

extern "C" int bnsn_gp19_load_header(const char* path)
{
    if (!path)
        return BNSN_ERR_ARG;
    FILE* f = fopen(path, "rb");
    if (!f)
        return BNSN_ERR_ARG;
    std::string s;
    char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0)
        s.append(buf, got);
    fclose(f);
    int dims[4];
    const char* dn[4] = {"GP19_nb_dims", "GP19_Ye_dims", "GP19_T_dims", "GP19_w_dims"};
    for (int k = 0; k < 4; ++k)
        if (!read_int(s, dn[k], &dims[k]) || dims[k] < 2 || dims[k] > (1 << 20))
            return BNSN_ERR_ARG;
    std::vector<double> ax[4], lognb, logw, data;
    const char* an[4] = {"GP19_nb_axis", "GP19_Ye_axis", "GP19_T_axis", "GP19_w_axis"};
    for (int k = 0; k < 4; ++k)
        if (!read_array(s, an[k], &ax[k]) || (int)ax[k].size() != dims[k])
            return BNSN_ERR_ARG;
    const bool has_lnb = read_array(s, "GP19_lognb_axis", &lognb);
    const bool has_lw  = read_array(s, "GP19_logw_axis", &logw);
    if ((has_lnb && (int)lognb.size() != dims[0]) || (has_lw && (int)logw.size() != dims[3]))
        return BNSN_ERR_ARG;
    const size_t nd = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
    if (!read_array(s, "GP19_data", &data) || data.size() != nd)
        return BNSN_ERR_ARG;
    return bnsn_gp19_set_table(dims, ax[0].data(), ax[1].data(), ax[2].data(), ax[3].data(),
                               has_lnb ? lognb.data() : nullptr, has_lw ? logw.data() : nullptr,
                               data.data());
}
