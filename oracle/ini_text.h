/*
 * INI text parsing with the reference's rules, shared by the C oracles
 * (mhd_oracle.c, hydro_oracle.c).  TEST INFRASTRUCTURE ONLY.
 * Restates inih ini.cpp:100-190 (line syntax, inline ';' comments after
 * whitespace, continuation lines), INIReader.cpp:40-117 (lower-cased
 * "section.name" keys) and ConfigMap.cpp:38-82 (getFloat through strtof,
 * getInteger through strtol base 0, getBool words).
 */
#ifndef PPKMHD_ORACLE_INI_TEXT_H
#define PPKMHD_ORACLE_INI_TEXT_H

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct
{
  char key[128];
  char val[256];
} ini_kv;

typedef struct
{
  ini_kv *kv;
  int     n, cap;
} ini_map;

static void
ini_set(ini_map *m, const char *section, const char *name, const char *value)
{
  char key[128];
  snprintf(key, sizeof key, "%s.%s", section, name);
  for (char *c = key; *c; ++c)
    *c = (char)tolower((unsigned char)*c); /* INIReader.cpp:100-105 */
  for (int q = 0; q < m->n; ++q)
    if (!strcmp(m->kv[q].key, key))
    {
      snprintf(m->kv[q].val, sizeof m->kv[q].val, "%s", value);
      return;
    }
  if (m->n == m->cap)
  {
    m->cap = m->cap ? 2 * m->cap : 32;
    m->kv = (ini_kv *)realloc(m->kv, (size_t)m->cap * sizeof(ini_kv));
  }
  snprintf(m->kv[m->n].key, sizeof m->kv[m->n].key, "%s", key);
  snprintf(m->kv[m->n].val, sizeof m->kv[m->n].val, "%s", value);
  m->n++;
}

static const char *
ini_get(const ini_map *m, const char *section, const char *name)
{
  char key[128];
  snprintf(key, sizeof key, "%s.%s", section, name);
  for (char *c = key; *c; ++c)
    *c = (char)tolower((unsigned char)*c);
  for (int q = 0; q < m->n; ++q)
    if (!strcmp(m->kv[q].key, key))
      return m->kv[q].val;
  return NULL;
}

static char *
str_rstrip(char *s)
{
  char *p = s + strlen(s);
  while (p > s && isspace((unsigned char)p[-1]))
    *--p = '\0';
  return s;
}

static char *
str_lskip(char *s)
{
  while (*s && isspace((unsigned char)*s))
    s++;
  return s;
}

/* first occurrence of c, or of a ';' that follows whitespace (inline comment) */
static char *
find_char_or_comment(char *s, char c)
{
  int ws = 0;
  while (*s && *s != c && !(ws && *s == ';'))
  {
    ws = isspace((unsigned char)*s);
    s++;
  }
  return s;
}

static void
ini_parse_text(ini_map *m, const char *text)
{
  char        section[64] = "";
  char        prev_name[64] = "";
  const char *p = text;
  while (*p)
  {
    char        line[512];
    const char *nl = strchr(p, '\n');
    size_t      len = nl ? (size_t)(nl - p) : strlen(p);
    if (len >= sizeof line)
      len = sizeof line - 1;
    memcpy(line, p, len);
    line[len] = '\0';
    p = nl ? nl + 1 : p + strlen(p);

    char *start = str_lskip(str_rstrip(line));
    if (*prev_name && *start && start > line)
    {
      ini_set(m, section, prev_name, start); /* continuation line */
    }
    else if (*start == ';' || *start == '#')
    {
    }
    else if (*start == '[')
    {
      char *end = find_char_or_comment(start + 1, ']');
      if (*end == ']')
      {
        *end = '\0';
        snprintf(section, sizeof section, "%s", start + 1);
        prev_name[0] = '\0';
      }
    }
    else if (*start)
    {
      char *end = find_char_or_comment(start, '=');
      if (*end == '=')
      {
        *end = '\0';
        char *name = str_rstrip(start);
        char *value = str_lskip(end + 1);
        end = find_char_or_comment(value, '\0');
        if (*end == ';')
          *end = '\0';
        str_rstrip(value);
        snprintf(prev_name, sizeof prev_name, "%s", name);
        ini_set(m, section, name, value);
      }
    }
  }
}

/* ConfigMap::getFloat: strtof, default value itself passed as float */
static double
ini_float(const ini_map *m, const char *s, const char *n, float def)
{
  const char *v = ini_get(m, s, n);
  if (!v)
    return (double)def;
  char *end;
  float f = strtof(v, &end);
  return end > v ? (double)f : (double)def;
}

/* INIReader::getInteger: strtol base 0 */
static long
ini_int(const ini_map *m, const char *s, const char *n, long def)
{
  const char *v = ini_get(m, s, n);
  if (!v)
    return def;
  char *end;
  long  x = strtol(v, &end, 0);
  return end > v ? x : def;
}

static const char *
ini_str(const ini_map *m, const char *s, const char *n, const char *def)
{
  const char *v = ini_get(m, s, n);
  return v ? v : def;
}

/* ConfigMap::getBool (ConfigMap.cpp:64-82): "1", "yes", "true", "on" and
 * "0", "no", "false", "off"; anything else keeps the default */
static inline int
ini_bool(const ini_map *m, const char *s, const char *n, int def)
{
  const char *v = ini_get(m, s, n);
  if (!v || !*v)
    return def;
  if (!strcmp(v, "1") || !strcmp(v, "yes") || !strcmp(v, "true") || !strcmp(v, "on"))
    return 1;
  if (!strcmp(v, "0") || !strcmp(v, "no") || !strcmp(v, "false") || !strcmp(v, "off"))
    return 0;
  return def;
}

#endif
