// .ini configuration map with the parsing rules of ppkMHD's ConfigMap /
// INIReader (src/utils/config/ConfigMap.{h,cpp}, src/utils/config/inih):
//   * "[section]" headers, "name = value" pairs, ';' or '#' comment lines,
//     ';' inline comments when preceded by whitespace, indented continuation
//     lines that replace the previous name's value;
//   * keys are "section.name" lower-cased, so lookups are case-insensitive;
//   * getFloat parses with strtof (the value is rounded to float),
//     getInteger with strtol base 0, getBool accepts 1/yes/true/on and
//     0/no/false/off.
#pragma once

#include <iosfwd>
#include <map>
#include <string>

class ConfigMap
{
public:
  //! Parse a file (ini_parse, ini.cpp:100-190).  ParseError() is -1 when the
  //! file cannot be opened, else the first bad line number or 0.
  explicit ConfigMap(const std::string & filename);
  //! Parse an in-memory buffer (ini_parse_buffer).
  ConfigMap(const char * buffer, int buffer_size);
  ConfigMap() = default;

  int
  ParseError() const
  {
    return m_error;
  }

  std::string
  getString(const std::string & section, const std::string & name,
            const std::string & default_value) const;
  void
  setString(const std::string & section, const std::string & name, const std::string & value);
  long
  getInteger(const std::string & section, const std::string & name, long default_value) const;
  void
  setInteger(const std::string & section, const std::string & name, long value);
  float
  getFloat(const std::string & section, const std::string & name, float default_value) const;
  void
  setFloat(const std::string & section, const std::string & name, float value);
  bool
  getBool(const std::string & section, const std::string & name, bool default_value) const;
  void
  setBool(const std::string & section, const std::string & name, bool value);

  const std::map<std::string, std::string> &
  values() const
  {
    return m_values;
  }

  friend std::ostream &
  operator<<(std::ostream & os, const ConfigMap & cfg);

private:
  static std::string
  makeKey(const std::string & section, const std::string & name);
  void
  parse_text(const std::string & text);

  std::map<std::string, std::string> m_values;
  int                                m_error = 0;
};
