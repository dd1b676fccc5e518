#include "ConfigMap.h"

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <ostream>
#include <sstream>

namespace
{

// whitespace trimming of one line, in place
char *
rstrip(char * s)
{
  char * p = s + std::strlen(s);
  while (p > s && std::isspace((unsigned char)p[-1]))
    *--p = '\0';
  return s;
}

char *
lskip(char * s)
{
  while (*s && std::isspace((unsigned char)*s))
    ++s;
  return s;
}

// first c, or first ';' that follows a whitespace character
char *
find_char_or_comment(char * s, char c)
{
  bool was_space = false;
  while (*s && *s != c && !(was_space && *s == ';'))
  {
    was_space = std::isspace((unsigned char)*s);
    ++s;
  }
  return s;
}

} // namespace

ConfigMap::ConfigMap(const std::string & filename)
{
  std::ifstream f(filename);
  if (!f)
  {
    m_error = -1;
    return;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  parse_text(ss.str());
}

ConfigMap::ConfigMap(const char * buffer, int buffer_size)
{
  parse_text(std::string(buffer, buffer + (buffer_size > 0 ? buffer_size : 0)));
}

std::string
ConfigMap::makeKey(const std::string & section, const std::string & name)
{
  std::string key = section + "." + name;
  for (char & c : key)
    c = (char)std::tolower((unsigned char)c);
  return key;
}

void
ConfigMap::parse_text(const std::string & text)
{
  std::string       section, prev_name;
  std::stringstream in(text);
  std::string       raw;
  int               lineno = 0;
  while (std::getline(in, raw))
  {
    ++lineno;
    std::string buf = raw; // writable copy
    char *      line = &buf[0];
    char *      start = lskip(rstrip(line));
    if (!prev_name.empty() && *start && start > line)
    {
      // indented line: continuation of the previous value
      m_values[makeKey(section, prev_name)] = start;
    }
    else if (*start == ';' || *start == '#')
    {
    }
    else if (*start == '[')
    {
      char * end = find_char_or_comment(start + 1, ']');
      if (*end == ']')
      {
        *end = '\0';
        section = start + 1;
        prev_name.clear();
      }
      else if (!m_error)
        m_error = lineno;
    }
    else if (*start)
    {
      char * end = find_char_or_comment(start, '=');
      if (*end == '=')
      {
        *end = '\0';
        char * name = rstrip(start);
        char * value = lskip(end + 1);
        end = find_char_or_comment(value, '\0');
        if (*end == ';')
          *end = '\0';
        rstrip(value);
        prev_name = name;
        m_values[makeKey(section, name)] = value;
      }
      else if (!m_error)
        m_error = lineno;
    }
  }
}

std::string
ConfigMap::getString(const std::string & section, const std::string & name,
                     const std::string & default_value) const
{
  auto it = m_values.find(makeKey(section, name));
  return it == m_values.end() ? default_value : it->second;
}

void
ConfigMap::setString(const std::string & section, const std::string & name,
                     const std::string & value)
{
  m_values[makeKey(section, name)] = value;
}

long
ConfigMap::getInteger(const std::string & section, const std::string & name,
                      long default_value) const
{
  const std::string v = getString(section, name, "");
  const char *      s = v.c_str();
  char *            end;
  const long        n = std::strtol(s, &end, 0);
  return end > s ? n : default_value;
}

void
ConfigMap::setInteger(const std::string & section, const std::string & name, long value)
{
  setString(section, name, std::to_string(value));
}

float
ConfigMap::getFloat(const std::string & section, const std::string & name,
                    float default_value) const
{
  const std::string v = getString(section, name, "");
  const char *      s = v.c_str();
  char *            end;
  const float       x = std::strtof(s, &end);
  return end > s ? x : default_value;
}

void
ConfigMap::setFloat(const std::string & section, const std::string & name, float value)
{
  std::stringstream ss;
  ss << value;
  setString(section, name, ss.str());
}

bool
ConfigMap::getBool(const std::string & section, const std::string & name, bool default_value) const
{
  const std::string v = getString(section, name, "");
  if (v.empty())
    return default_value;
  if (v == "1" || v == "yes" || v == "true" || v == "on")
    return true;
  if (v == "0" || v == "no" || v == "false" || v == "off")
    return false;
  return default_value;
}

void
ConfigMap::setBool(const std::string & section, const std::string & name, bool value)
{
  setString(section, name, value ? "true" : "false");
}

std::ostream &
operator<<(std::ostream & os, const ConfigMap & cfg)
{
  for (const auto & kv : cfg.m_values)
    os << kv.first << " = " << kv.second << "\n";
  return os;
}
