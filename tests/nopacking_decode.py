"""extract (pir/extract.rs:16-45) for unpacked responses, restated for the tests: each
column ciphertext decrypts with the RLWE secret (rlwe/enc.rs:91-107) to the column's value
at coefficient 0, rounded by delta = q / p; the 16-bit values give the entry bytes
(encode_db.rs reconstruct_entry)."""


def coeff0_decrypt(a, b, s, q, p):
    n = len(a)
    acc = int(a[0]) * int(s[0])
    for i in range(1, n):
        acc -= int(a[i]) * int(s[n - i])  # X^n = -1
    noisy = (acc + int(b[0])) % q
    delta = q // p
    return ((noisy + delta // 2) // delta) % p


def extract(column_ciphertexts, secret, q, p, entry_size):
    values = [coeff0_decrypt(a, b, secret, q, p) for a, b in column_ciphertexts]
    entry = bytearray(entry_size)
    for j, v in enumerate(values):
        if 2 * j < entry_size:
            entry[2 * j] = v & 0xFF
        if 2 * j + 1 < entry_size:
            entry[2 * j + 1] = (v >> 8) & 0xFF
    return bytes(entry)
