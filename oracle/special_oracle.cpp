// special_modulus restatement: filled in below.
