/*
 * json.h - a small strict JSON reader (RFC 8259) for graph descriptions:
 * objects, arrays, strings with escapes (\uXXXX to UTF-8, surrogate pairs
 * included), numbers, true/false/null. The tree lives in one arena freed by
 * json_free.
 */
#ifndef UFOIR_JSON_H
#define UFOIR_JSON_H

#include <stddef.h>

typedef enum { JSON_NULL, JSON_BOOL, JSON_NUMBER, JSON_STRING, JSON_ARRAY, JSON_OBJECT } json_type;

typedef struct json_value json_value;
struct json_value {
    json_type type;
    double number;          /* JSON_NUMBER; JSON_BOOL as 0 / 1 */
    const char *string;     /* JSON_STRING (NUL-terminated, UTF-8) */
    size_t count;           /* members of an object / elements of an array */
    const char **keys;      /* JSON_OBJECT: member names */
    json_value **items;     /* JSON_OBJECT / JSON_ARRAY: values */
};

typedef struct json_doc json_doc;

/* Parses text[0, len). On error returns NULL and writes a message with the
 * line and column to err. */
json_doc *json_parse(const char *text, size_t len, char *err, size_t errlen);
const json_value *json_root(const json_doc *doc);
void json_free(json_doc *doc);

/* Member of an object by exact name, or NULL. */
const json_value *json_get(const json_value *obj, const char *key);

#endif
