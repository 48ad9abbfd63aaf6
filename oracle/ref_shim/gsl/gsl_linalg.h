/* empty stand-in: the hot-path sources include this header but call nothing in it */
